// Context runtime of liblra: errors, device workspace arena, launch hooks.

#include <cstdlib>
#include <cstdio>
#include <cstring>
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

}  // namespace lra
