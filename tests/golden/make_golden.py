"""Generate the golden fixtures of tests/golden/ (run in the build container).

The reference is Julia and cannot run here, so its outputs are pinned
through the native routine it calls: the pivoted-QR block loop of
geqp3_adap! (src/pqr.jl:361-418) is driven around the real LAPACK xLAQPS
exported by numpy's bundled OpenBLAS -- the routine the reference `ccall`s
(src/lapack.jl:117-139).  Dense post-processing uses numpy's LAPACK
(geqrf / gesdd / syevd), as the reference uses Julia's stdlib LAPACK.

Sketch inputs are the "lattice Gaussian" stream every test uses: N(0,1)
draws of numpy.random.default_rng(seed) rounded to the nearest multiple of
1/32 and clipped to [-127/32, 127/32], stored as int8 (value = int8 / 32).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def lattice_gauss(seed: int, n: int) -> np.ndarray:
    g = np.random.default_rng(seed).standard_normal(n)
    return np.clip(np.rint(g * 32.0), -127, 127).astype(np.int8)


def laqps_cases():
    """Pivoted QR cases (B, options) covering the reference's branches."""
    rng = np.random.default_rng(11)
    cases = []
    # decaying spectrum, short-fat (the sketch shape)
    B = rng.standard_normal((40, 120)) @ np.diag(np.exp(-np.arange(120) / 1.5))
    cases.append(("decay_40x120", B, 1e-10, -1))
    # tall, full rank
    cases.append(("tall_70x30", rng.standard_normal((70, 30)), 1e-14, -1))
    # duplicate and zero columns (pivot ties: first index wins)
    C = rng.standard_normal((30, 50))
    C[:, 7] = C[:, 3]
    C[:, 20] = 0.0
    C[:, 33] = C[:, 3]
    cases.append(("ties_30x50", C, 1e-12, -1))
    # strong cancellation: triggers the norm recomputation (lsticc) branch
    base = rng.standard_normal((60, 6))
    D = base @ rng.standard_normal((6, 90)) + 1e-13 * rng.standard_normal((60, 90))
    cases.append(("cancel_60x90", D, 1e-10, -1))
    # fixed rank option
    cases.append(("rank5_40x80", rng.standard_normal((40, 80)), 0.0, 5))
    # Hilbert block
    cases.append(("hilb_48x200", O.hilb(48, 200), 1e-13, -1))
    return cases


def main():
    out = {}
    for name, B, rtol, rank in laqps_cases():
        for dt in (np.float64, np.float32):
            tag = f"{name}_{np.dtype(dt).name}"
            Bf = np.asfortranarray(B.astype(dt))
            opts = O.Opts(rtol=max(rtol, 1e-6) if dt == np.float32 else rtol, rank=rank)
            opts = opts.for_dtype(dt)
            W = Bf.copy(order="F")
            p, tau, k = O.geqp3_adap(W, opts, backend="lapack")
            out[f"qr/{tag}/B"] = Bf
            out[f"qr/{tag}/rtol"] = np.array(opts.rtol)
            out[f"qr/{tag}/rank"] = np.array(rank)
            out[f"qr/{tag}/p"] = p
            out[f"qr/{tag}/k"] = np.array(k)
            out[f"qr/{tag}/R"] = np.triu(W[:k, :])
            out[f"qr/{tag}/tau"] = tau[:k]
    np.savez_compressed(os.path.join(HERE, "laqps_cases.npz"), **out)

    # Hilbert 1024 idfact (the reference README's CPU-sized case), rtol 1e-12 and the
    # default 5 eps; 40 x 1024 lattice-Gaussian sketch from seed 0.
    A = O.hilb(1024)
    s = lattice_gauss(0, 40 * 1024 * 2)
    hil = {"stream": s}
    for tag, rtol in (("1e-12", 1e-12), ("default", None)):
        rs = O.RandStream(gauss=s.astype(np.float64) / 32.0)
        V = O.idfact("n", A, O.Opts(rtol=rtol), rs, backend="lapack")
        hil[f"{tag}/k"] = np.array(V["k"])
        hil[f"{tag}/sk"] = V["sk"]
        hil[f"{tag}/rd"] = V["rd"]
        hil[f"{tag}/T"] = V["T"]
        hil[f"{tag}/nsteps"] = np.array(V["nsteps"])
        E = O.id_matrix("n", A, V)
        hil[f"{tag}/relerr2"] = np.array(np.linalg.norm(A - E, 2) / np.linalg.norm(A, 2))
    np.savez_compressed(os.path.join(HERE, "hilbert1024_id.npz"), **hil)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
