// Context runtime of liblra: errors, device workspace arena, launch hooks.

#include <dlfcn.h>

#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <mutex>
#include <set>
#include <utility>

#include "internal.hpp"

namespace lra {

void fail(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw Error{status, buf};
}

void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(LRA_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
  }
  fail(LRA_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

void post_launch(lra_ctx* ctx, const char* name) {
  count_launch(ctx);
  ++ctx->launches_by_name[name];
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fail(LRA_ECUDA, "launch of %s: %s", name, cudaGetErrorString(e));
}

static constexpr size_t kAlign = 256;

void Arena::free_all(cudaStream_t stream) {
  cudaStreamSynchronize(stream);
  for (auto& c : chunks_) cudaFree(c.base);
  chunks_.clear();
  cur_ = 0;
}

Arena::~Arena() {
  for (auto& c : chunks_) cudaFree(c.base);
}

void* Arena::alloc(size_t bytes) {
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  if (bytes == 0) bytes = kAlign;
  while (cur_ < chunks_.size()) {
    Chunk& c = chunks_[cur_];
    if (c.used + bytes <= c.cap) {
      void* p = c.base + c.used;
      c.used += bytes;
      return p;
    }
    if (cur_ + 1 < chunks_.size()) {
      ++cur_;
      chunks_[cur_].used = 0;
      continue;
    }
    break;
  }
  size_t want = bytes;
  size_t have = capacity();
  if (have > want) want = have;  // grow geometrically
  if (want < (64u << 20)) want = 64u << 20;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess && want > bytes) {
    cudaGetLastError();
    want = bytes;
    e = cudaMalloc(&p, want);
  }
  check_cuda(e, "cudaMalloc(workspace)");
  chunks_.push_back(Chunk{static_cast<char*>(p), want, bytes});
  cur_ = chunks_.size() - 1;
  return p;
}

ArenaMark Arena::mark() const {
  if (chunks_.empty()) return ArenaMark{0, 0};
  return ArenaMark{cur_, chunks_[cur_].used};
}

void Arena::release(ArenaMark m) {
  if (chunks_.empty()) return;
  for (size_t i = m.chunk + 1; i < chunks_.size() && i <= cur_; ++i) chunks_[i].used = 0;
  cur_ = m.chunk;
  chunks_[cur_].used = m.used;
}

void Arena::reset(cudaStream_t stream) {
  if (chunks_.size() > 1) {
    size_t total = capacity();
    cudaStreamSynchronize(stream);
    for (auto& c : chunks_) cudaFree(c.base);
    chunks_.clear();
    void* p = nullptr;
    check_cuda(cudaMalloc(&p, total), "cudaMalloc(workspace)");
    chunks_.push_back(Chunk{static_cast<char*>(p), total, 0});
  }
  cur_ = 0;
  if (!chunks_.empty()) chunks_[0].used = 0;
}

size_t Arena::capacity() const {
  size_t s = 0;
  for (auto& c : chunks_) s += c.cap;
  return s;
}

void raise_smem_limit(lra_ctx* ctx, const void* kernel) {
  // the attribute holds a fixed value per kernel and device: set it once
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({kernel, ctx->device})) return;
  }
  int optin = 0;
  check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device),
             "cudaDeviceGetAttribute(MaxSharedMemoryPerBlockOptin)");
  cudaFuncAttributes fa;
  check_cuda(cudaFuncGetAttributes(&fa, kernel), "cudaFuncGetAttributes");
  check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes),
             "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)");
  std::lock_guard<std::mutex> lk(mu);
  done.insert({kernel, ctx->device});
}

bool trace_on() {
  static const bool on = [] {
    const char* e = std::getenv("LRA_TRACE");
    return e && *e && *e != '0';
  }();
  return on;
}

// ---- tuning table -------------------------------------------------------------------
//
// Text, one entry per line ("#" starts a comment):
//   tc_tile_n <f32|f64> <log2 order> <32|64|96>
//   qr_seq_len <rows>
//   srft_wide <log2 l'> <0|1>
//   qr_steps <1..8>
//   qr_sms <SMs a pivoted-QR launch may take; 0: all>
//   tc_split <most K parts of the tensor-core sketch; 0: as many as fill the SMs>
//   jacobi_jb <columns per FP32 Jacobi block: 4, 8, 16, 32; 0: by size>
//   jacobi_cluster <largest cluster of the in-cluster FP32 Jacobi, 2..16; 0: largest schedulable; 1: off>
//   trsm_inv <0: FP64 triangular solves on the tensor-core path by the explicit inverse; 1: substitution>
//   gram_start <cosine x 1e4 where the FP32 Jacobi sweeps stop; 0: min(3e-2, 12 / n)>
// lowrankapprox/autotune.py writes it from its sweeps; unknown keys and
// out-of-range values are ignored, so an old table never breaks a newer
// library.

static void tuning_defaults(lra_tuning* t) {
  for (auto& row : t->tc_tile_n)
    for (int& v : row) v = 96;
  t->qr_seq_len = 96;
  for (int lb = 0; lb <= 10; ++lb) t->srft_wide[lb] = (lb >= 7 && lb <= 10) ? 1 : 0;
  t->qr_steps = 8;
  t->qr_sms = 0;
  t->tc_split = 0;
  t->jacobi_jb = 0;
  t->jacobi_cluster = 0;
  t->trsm_inv = 0;
  t->gram_start = 0;
}

bool set_tuning(lra_tuning* t, const char* key, int64_t index, int64_t value) {
  if (!std::strcmp(key, "tc_tile_n")) {
    if (index < 0 || index >= 32 || (value != 32 && value != 64 && value != 96)) return false;
    t->tc_tile_n[index / 16][index % 16] = (int)value;
    return true;
  }
  if (!std::strcmp(key, "qr_seq_len")) {
    if (value < 0 || value > 4096) return false;
    t->qr_seq_len = (int)value;
    return true;
  }
  if (!std::strcmp(key, "srft_wide")) {
    if (index < 0 || index > 10 || (value != 0 && value != 1)) return false;
    t->srft_wide[index] = (int)value;
    return true;
  }
  if (!std::strcmp(key, "qr_steps")) {
    if (value < 1 || value > 8) return false;
    t->qr_steps = (int)value;
    return true;
  }
  if (!std::strcmp(key, "qr_sms")) {
    if (value < 0 || value > 4096) return false;
    t->qr_sms = (int)value;
    return true;
  }
  if (!std::strcmp(key, "tc_split")) {
    if (value < 0 || value > 4096) return false;
    t->tc_split = (int)value;
    return true;
  }
  if (!std::strcmp(key, "gram_start")) {
    if (value < 0 || value > 5000) return false;
    t->gram_start = (int)value;
    return true;
  }
  if (!std::strcmp(key, "trsm_inv")) {
    if (value != 0 && value != 1) return false;
    t->trsm_inv = (int)value;
    return true;
  }
  if (!std::strcmp(key, "jacobi_cluster")) {
    if (value < 0 || value > 16) return false;
    t->jacobi_cluster = (int)value;
    return true;
  }
  if (!std::strcmp(key, "jacobi_jb")) {
    if (value != 0 && value != 4 && value != 8 && value != 16 && value != 32) return false;
    t->jacobi_jb = (int)value;
    return true;
  }
  return false;
}

static std::string library_dir() {
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&tuning_defaults), &info) && info.dli_fname) {
    std::string p = info.dli_fname;
    const size_t slash = p.rfind('/');
    if (slash != std::string::npos) return p.substr(0, slash);
  }
  return ".";
}

void load_tuning(lra_tuning* t, std::string* source) {
  tuning_defaults(t);
  *source = "defaults";
  const char* env = std::getenv("LRA_TUNING");
  const std::string path = env && *env ? std::string(env) : library_dir() + "/tuning_gb300.txt";
  std::ifstream f(path);
  if (!f) return;
  std::string line;
  int used = 0;
  while (std::getline(f, line)) {
    const size_t hash = line.find('#');
    if (hash != std::string::npos) line.resize(hash);
    std::istringstream in(line);
    std::string key;
    if (!(in >> key)) continue;
    if (key == "tc_tile_n") {
      std::string dt;
      int64_t lb = -1, v = 0;
      if (in >> dt >> lb >> v) used += set_tuning(t, "tc_tile_n", (dt == "f64" ? 16 : 0) + lb, v);
    } else if (key == "qr_seq_len") {
      int64_t v = 0;
      if (in >> v) used += set_tuning(t, "qr_seq_len", 0, v);
    } else if (key == "srft_wide") {
      int64_t lb = -1, v = 0;
      if (in >> lb >> v) used += set_tuning(t, "srft_wide", lb, v);
    } else if (key == "qr_steps" || key == "qr_sms" || key == "tc_split" || key == "jacobi_jb" ||
               key == "jacobi_cluster" || key == "trsm_inv" || key == "gram_start") {
      int64_t v = 0;
      if (in >> v) used += set_tuning(t, key.c_str(), 0, v);
    }
  }
  *source = path + " (" + std::to_string(used) + " entries)";
}

std::string tuning_text(const lra_tuning& t) {
  std::ostringstream o;
  for (int d = 0; d < 2; ++d)
    for (int lb = 0; lb < 16; ++lb) o << "tc_tile_n " << (d ? "f64 " : "f32 ") << lb << ' ' << t.tc_tile_n[d][lb] << '\n';
  o << "qr_seq_len " << t.qr_seq_len << '\n';
  for (int lb = 0; lb <= 10; ++lb) o << "srft_wide " << lb << ' ' << t.srft_wide[lb] << '\n';
  o << "qr_steps " << t.qr_steps << '\n';
  o << "qr_sms " << t.qr_sms << '\n';
  o << "tc_split " << t.tc_split << '\n';
  o << "jacobi_jb " << t.jacobi_jb << '\n';
  o << "jacobi_cluster " << t.jacobi_cluster << '\n';
  o << "trsm_inv " << t.trsm_inv << '\n';
  o << "gram_start " << t.gram_start << '\n';
  return o.str();
}

}  // namespace lra
