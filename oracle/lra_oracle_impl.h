/*
 * Type-generic body of the CPU oracle (included twice by lra_oracle.c, once
 * with REAL = double / SFX = d and once with REAL = float / SFX = s).
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker that the CUDA path is
 * compared with; the product never links or calls it.
 *
 * It restates, in plain C:
 *   - LAPACK xNRM2 / xLAPY2 / xLARFG / xLAQPS (the published reference
 *     LAPACK algorithms; the reference reaches xLAQPS through the `ccall` in
 *     src/lapack.jl:117-139, libblastrampoline -> OpenBLAS, version unpinned
 *     because Project.toml ships no Manifest);
 *   - geqp3_adap! / geqp3_adap_main! (src/pqr.jl:348-418);
 *   - maxdet_t, T = R11 \ R12 (src/pqr.jl:438-442);
 *   - maxdet_swapcols! / maxdet_update! (src/pqr.jl:445-501).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(CAT(ora_, SFX), name)

/* xNRM2, classic scaled sum of squares */
REAL FN(nrm2)(int64_t n, const REAL* x, int64_t incx) {
  if (n < 1) return (REAL)0;
  if (n == 1) return (REAL)fabs((double)x[0]);
  REAL scale = 0, ssq = 1;
  for (int64_t i = 0; i < n; ++i) {
    REAL v = x[i * incx];
    if (v != 0) {
      REAL a = (REAL)fabs((double)v);
      if (scale < a) {
        REAL r = scale / a;
        ssq = 1 + ssq * r * r;
        scale = a;
      } else {
        REAL r = a / scale;
        ssq += r * r;
      }
    }
  }
  return scale * (REAL)sqrt((double)ssq);
}

/* xLAPY2: sqrt(x^2 + y^2) without needless overflow */
static REAL FN(lapy2)(REAL x, REAL y) {
  if (isnan((double)x)) return x;
  if (isnan((double)y)) return y;
  REAL xa = (REAL)fabs((double)x), ya = (REAL)fabs((double)y);
  REAL w = xa > ya ? xa : ya;
  REAL z = xa > ya ? ya : xa;
  if (z == 0 || w > REAL_MAX) return w;
  REAL q = z / w;
  return w * (REAL)sqrt((double)(1 + q * q));
}

/* xLARFG: H * [alpha; x] = [beta; 0], H = I - tau [1; v][1; v]^T */
void FN(larfg)(int64_t n, REAL* alpha, REAL* x, int64_t incx, REAL* tau) {
  if (n <= 1) {
    *tau = 0;
    return;
  }
  REAL xnorm = FN(nrm2)(n - 1, x, incx);
  if (xnorm == 0) {
    *tau = 0;
    return;
  }
  REAL beta = -(REAL)copysign((double)FN(lapy2)(*alpha, xnorm), (double)*alpha);
  const REAL safmin = REAL_SAFMIN / REAL_EPS;
  int knt = 0;
  if (fabs((double)beta) < safmin) {
    const REAL rsafmn = 1 / safmin;
    do {
      ++knt;
      for (int64_t i = 0; i < n - 1; ++i) x[i * incx] *= rsafmn;
      beta *= rsafmn;
      *alpha *= rsafmn;
    } while (fabs((double)beta) < safmin && knt < 20);
    xnorm = FN(nrm2)(n - 1, x, incx);
    beta = -(REAL)copysign((double)FN(lapy2)(*alpha, xnorm), (double)*alpha);
  }
  *tau = (beta - *alpha) / beta;
  REAL scal = 1 / (*alpha - beta);
  for (int64_t i = 0; i < n - 1; ++i) x[i * incx] *= scal;
  for (int j = 0; j < knt; ++j) beta *= safmin;
  *alpha = beta;
}

/*
 * xLAQPS: one block of column-pivoted Householder QR with lazy (F-based)
 * trailing updates and early exit when a partial norm must be recomputed.
 * Arguments and indexing follow the Fortran routine (1-based JPVT, A(i,j)
 * at a[(i-1) + (j-1)*lda]); ldf >= n.
 */
void FN(laqps)(int64_t m, int64_t n, int64_t offset, int64_t nb, int64_t* kb,
               REAL* a, int64_t lda, int64_t* jpvt, REAL* tau, REAL* vn1,
               REAL* vn2, REAL* auxv, REAL* f, int64_t ldf) {
#define A_(i, j) a[((i)-1) + ((j)-1) * lda]
#define F_(i, j) f[((i)-1) + ((j)-1) * ldf]
  const int64_t lastrk = m < n + offset ? m : n + offset;
  int64_t lsticc = 0;
  int64_t k = 0;
  const REAL tol3z = (REAL)sqrt((double)REAL_EPS);
  while (k < nb && lsticc == 0) {
    ++k;
    const int64_t rk = offset + k;
    /* pivot: first index of the maximum of vn1(k:n) (IxAMAX) */
    int64_t pvt = k;
    {
      REAL best = (REAL)fabs((double)vn1[k - 1]);
      for (int64_t j = k + 1; j <= n; ++j) {
        REAL v = (REAL)fabs((double)vn1[j - 1]);
        if (v > best) {
          best = v;
          pvt = j;
        }
      }
    }
    if (pvt != k) {
      for (int64_t i = 1; i <= m; ++i) {
        REAL t = A_(i, pvt);
        A_(i, pvt) = A_(i, k);
        A_(i, k) = t;
      }
      for (int64_t j = 1; j <= k - 1; ++j) {
        REAL t = F_(pvt, j);
        F_(pvt, j) = F_(k, j);
        F_(k, j) = t;
      }
      int64_t it = jpvt[pvt - 1];
      jpvt[pvt - 1] = jpvt[k - 1];
      jpvt[k - 1] = it;
      vn1[pvt - 1] = vn1[k - 1];
      vn2[pvt - 1] = vn2[k - 1];
    }
    /* A(rk:m,k) -= A(rk:m,1:k-1) * F(k,1:k-1)^T */
    if (k > 1) {
      for (int64_t j = 1; j <= k - 1; ++j) {
        REAL t = -F_(k, j);
        if (t != 0)
          for (int64_t i = rk; i <= m; ++i) A_(i, k) += t * A_(i, j);
      }
    }
    /* reflector H(k) */
    if (rk < m)
      FN(larfg)(m - rk + 1, &A_(rk, k), &A_(rk + 1, k), 1, &tau[k - 1]);
    else
      FN(larfg)(1, &A_(rk, k), &A_(rk, k), 1, &tau[k - 1]);
    const REAL akk = A_(rk, k);
    A_(rk, k) = 1;
    /* F(k+1:n,k) = tau(k) * A(rk:m,k+1:n)^T * A(rk:m,k) */
    if (k < n) {
      for (int64_t j = k + 1; j <= n; ++j) {
        REAL s = 0;
        for (int64_t i = rk; i <= m; ++i) s += A_(i, j) * A_(i, k);
        F_(j, k) = tau[k - 1] * s;
      }
    }
    for (int64_t j = 1; j <= k; ++j) F_(j, k) = 0;
    /* F(1:n,k) -= tau(k) * F(1:n,1:k-1) * A(rk:m,1:k-1)^T * A(rk:m,k) */
    if (k > 1) {
      for (int64_t j = 1; j <= k - 1; ++j) {
        REAL s = 0;
        for (int64_t i = rk; i <= m; ++i) s += A_(i, j) * A_(i, k);
        auxv[j - 1] = -tau[k - 1] * s;
      }
      for (int64_t j = 1; j <= k - 1; ++j) {
        REAL t = auxv[j - 1];
        if (t != 0)
          for (int64_t i = 1; i <= n; ++i) F_(i, k) += t * F_(i, j);
      }
    }
    /* A(rk,k+1:n) -= A(rk,1:k) * F(k+1:n,1:k)^T */
    if (k < n) {
      for (int64_t j = 1; j <= k; ++j) {
        REAL t = -A_(rk, j);
        if (t != 0)
          for (int64_t i = k + 1; i <= n; ++i) A_(rk, i) += t * F_(i, j);
      }
    }
    /* downdate the partial column norms */
    if (rk < lastrk) {
      for (int64_t j = k + 1; j <= n; ++j) {
        if (vn1[j - 1] != 0) {
          REAL temp = (REAL)fabs((double)A_(rk, j)) / vn1[j - 1];
          temp = (1 + temp) * (1 - temp);
          if (temp < 0) temp = 0;
          REAL r = vn1[j - 1] / vn2[j - 1];
          REAL temp2 = temp * r * r;
          if (temp2 <= tol3z) {
            vn2[j - 1] = (REAL)lsticc;
            lsticc = j;
          } else {
            vn1[j - 1] = vn1[j - 1] * (REAL)sqrt((double)temp);
          }
        }
      }
    }
    A_(rk, k) = akk;
  }
  *kb = k;
  const int64_t rk = offset + k;
  /* A(rk+1:m,kb+1:n) -= A(rk+1:m,1:kb) * F(kb+1:n,1:kb)^T */
  {
    int64_t lim = n < m - offset ? n : m - offset;
    if (k < lim) {
      for (int64_t j = k + 1; j <= n; ++j)
        for (int64_t l = 1; l <= k; ++l) {
          REAL t = -F_(j, l);
          if (t != 0)
            for (int64_t i = rk + 1; i <= m; ++i) A_(i, j) += t * A_(i, l);
        }
    }
  }
  /* recompute the flagged norms (linked list threaded through vn2) */
  while (lsticc > 0) {
    int64_t itemp = (int64_t)llround((double)vn2[lsticc - 1]);
    vn1[lsticc - 1] = FN(nrm2)(m - rk, &A_(rk + 1, lsticc), 1);
    vn2[lsticc - 1] = vn1[lsticc - 1];
    lsticc = itemp;
  }
#undef A_
#undef F_
}

typedef void (*FN(laqps_fn))(int64_t, int64_t, int64_t, int64_t, int64_t*,
                             REAL*, int64_t, int64_t*, REAL*, REAL*, REAL*,
                             REAL*, REAL*, int64_t);

/*
 * geqp3_adap! (src/pqr.jl:348-359) + geqp3_adap_main! (src/pqr.jl:361-418).
 * jpvt (n) receives the 1-based permutation, tau (>= min(m,n)) the reflector
 * scalars, *k_out the rank.  Returns 0.
 */
int FN(geqp3_adap)(int64_t m, int64_t n, REAL* a, int64_t lda, int64_t* jpvt,
                   REAL* tau, double atol, double rtol, int64_t rank,
                   int64_t nbopt, int64_t* k_out) {
  for (int64_t j = 0; j < n; ++j) jpvt[j] = j + 1;
  const int64_t l = m < n ? m : n;
  int64_t k = (rank < 0 || rank > l) ? l : rank;
  if (k <= 0) {
    *k_out = k < 0 ? 0 : k;
    return 0;
  }
  const int64_t nb = nbopt < k ? nbopt : k;
  REAL* vn1 = (REAL*)malloc(sizeof(REAL) * (size_t)n);
  REAL* vn2 = (REAL*)malloc(sizeof(REAL) * (size_t)n);
  REAL* auxv = (REAL*)malloc(sizeof(REAL) * (size_t)nb);
  REAL* f = (REAL*)calloc((size_t)(n + 1) * (size_t)nb, sizeof(REAL));
  double maxnrm = 0;
  for (int64_t j = 0; j < n; ++j) {
    vn1[j] = vn2[j] = FN(nrm2)(m, a + j * lda, 1);
    if ((double)vn1[j] > maxnrm) maxnrm = (double)vn1[j];
  }
  const double ptol = atol > rtol * maxnrm ? atol : rtol * maxnrm;
  int64_t j = 1;
  int64_t result = k;
  while (j <= k) {
    int64_t jb = nb < k - j + 1 ? nb : k - j + 1;
    int64_t fjb = 0;
    FN(laqps)(m, n - j + 1, j - 1, jb, &fjb, a + (j - 1) * lda, lda,
              jpvt + (j - 1), tau + (j - 1), vn1 + (j - 1), vn2 + (j - 1), auxv,
              f, n - j + 1 > 1 ? n - j + 1 : 1);
    int64_t jn = j + fjb;
    if (fabs((double)a[(jn - 2) + (jn - 2) * lda]) <= ptol) {
      int found = 0;
      for (int64_t i = j; i <= jn - 1; ++i) {
        if (fabs((double)a[(i - 1) + (i - 1) * lda]) <= ptol) {
          result = i - 1;
          found = 1;
          break;
        }
      }
      if (found) break;
    }
    j = jn;
  }
  free(vn1);
  free(vn2);
  free(auxv);
  free(f);
  *k_out = result;
  return 0;
}

/* maxdet_t: T = triu(R)[1:k,1:k] \ R[1:k,k+1:n]; R is k x n (ldr), T is
   k x (n-k) (ldt).  Column-by-column back substitution.                    */
int FN(maxdet_t)(int64_t k, int64_t n, const REAL* r, int64_t ldr, REAL* t,
                 int64_t ldt) {
  for (int64_t c = 0; c < n - k; ++c) {
    REAL* x = t + c * ldt;
    const REAL* b = r + (k + c) * ldr;
    for (int64_t i = 0; i < k; ++i) x[i] = b[i];
    for (int64_t i = k - 1; i >= 0; --i) {
      x[i] /= r[i + i * ldr];
      REAL xi = x[i];
      if (xi != 0)
        for (int64_t q = 0; q < i; ++q) x[q] -= xi * r[q + i * ldr];
    }
  }
  return 0;
}

#undef FN
#undef CAT
#undef CAT2
