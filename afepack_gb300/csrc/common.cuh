// Shared host/device utilities of the afepack_gb300 library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/afepack_gb300.h"

namespace afp {

// ---------------------------------------------------------------- errors
struct Error {
  afp_status status;
  std::string msg;
};

void set_last_error(const std::string& msg);

[[noreturn]] inline void fail(afp_status s, const std::string& msg) { throw Error{s, msg}; }

#define AFP_CUDA(expr)                                                                  \
  do {                                                                                  \
    cudaError_t afp_e_ = (expr);                                                        \
    if (afp_e_ != cudaSuccess)                                                          \
      ::afp::fail(afp_e_ == cudaErrorMemoryAllocation ? AFP_ERR_OUT_OF_MEMORY : AFP_ERR_CUDA, \
                  std::string(#expr) + " -> " + cudaGetErrorString(afp_e_) + " (" + __FILE__ + \
                      ":" + std::to_string(__LINE__) + ")");                            \
  } while (0)

#define AFP_REQUIRE(cond, status, msg)                          \
  do {                                                          \
    if (!(cond)) ::afp::fail((status), std::string(msg));       \
  } while (0)

// Runs f and converts exceptions into a status (the C-ABI boundary).
template <class F>
afp_status guarded(F&& f) {
  try {
    f();
    return AFP_OK;
  } catch (const Error& e) {
    set_last_error(e.msg);
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return AFP_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return AFP_ERR_INVALID;
  }
}

// Counts this library's kernel launches (reported by afp_context_launch_count).
struct LaunchCounter {
  int64_t n = 0;
};

}  // namespace afp

// ---------------------------------------------------------------- context
struct afp_context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  afp::LaunchCounter launches;
  // device-side scalars for reductions (lives as long as the context)
  double* d_scalars = nullptr;
  double* h_scalars = nullptr;  // pinned mirror
  // per-context reduction scratch: block partials and the retire counter of
  // the last-block-reduces pattern, so that contexts on different streams
  // never share them
  double* d_partials = nullptr;
  unsigned* d_retire = nullptr;
  // device bytes held through DevBuf on this context and their high-water
  // mark (the server measures each request's footprint with them)
  mutable std::atomic<int64_t> dev_bytes{0}, dev_peak{0};
};

namespace afp {

// Makes the context's device current for the calling thread.
void bind(const afp_context* ctx);

// Adds d bytes to the context's DevBuf total and raises its high-water mark.
inline void note_device_bytes(const afp_context* ctx, int64_t d) {
  const int64_t v = ctx->dev_bytes.fetch_add(d, std::memory_order_relaxed) + d;
  int64_t p = ctx->dev_peak.load(std::memory_order_relaxed);
  while (v > p && !ctx->dev_peak.compare_exchange_weak(p, v, std::memory_order_relaxed)) {
  }
}

// -------------------------------------------------------------- device buffer
// Stream-ordered device allocation (cudaMallocAsync on the context stream).
template <class T>
class DevBuf {
 public:
  DevBuf() = default;
  DevBuf(const afp_context* ctx, size_t n) { alloc(ctx, n); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { swap(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      swap(o);
    }
    return *this;
  }
  ~DevBuf() { release(); }

  void alloc(const afp_context* ctx, size_t n) {
    release();
    ctx_ = ctx;
    n_ = n;
    if (n == 0) return;
    void* p = nullptr;
    AFP_CUDA(cudaMallocAsync(&p, n * sizeof(T), ctx->stream));
    p_ = static_cast<T*>(p);
    note_device_bytes(ctx, (int64_t)(n * sizeof(T)));
  }
  void release() noexcept {
    if (p_ != nullptr && ctx_ != nullptr) {
      cudaFreeAsync(p_, ctx_->stream);
      note_device_bytes(ctx_, -(int64_t)(n_ * sizeof(T)));
    }
    p_ = nullptr;
    n_ = 0;
  }
  void zero() {
    if (n_) AFP_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), ctx_->stream));
  }
  void upload(const T* src, size_t n) {
    if (n) AFP_CUDA(cudaMemcpyAsync(p_, src, n * sizeof(T), cudaMemcpyDefault, ctx_->stream));
  }
  void download(T* dst, size_t n) const {
    if (n) AFP_CUDA(cudaMemcpyAsync(dst, p_, n * sizeof(T), cudaMemcpyDefault, ctx_->stream));
  }
  T* get() const { return p_; }
  size_t size() const { return n_; }
  void swap(DevBuf& o) noexcept {
    std::swap(p_, o.p_);
    std::swap(n_, o.n_);
    std::swap(ctx_, o.ctx_);
  }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
  const afp_context* ctx_ = nullptr;
};

// Host <-> device copy of any pointer pair (unified addressing).
void copy(const afp_context* ctx, void* dst, const void* src, size_t bytes);
void sync(const afp_context* ctx);
// Raises AFP_ERR_CUDA if a kernel launch failed.
void check_launch(const afp_context* ctx, const char* what);

// Exclusive scan of n int32 counts into out[0..n] (out[n] = total); returns total.
int64_t exclusive_scan(const afp_context* ctx, const int* counts, int* out, int64_t n);

// --------------------------------------------------------------- CSR pattern
struct Pattern {
  int64_t m = 0, n = 0, nnz = 0;
  DevBuf<int> rowptr;  // m+1
  DevBuf<int> cols;    // nnz
};

}  // namespace afp

struct afp_matrix {
  afp_context* ctx = nullptr;
  std::shared_ptr<afp::Pattern> pat;
  afp::DevBuf<double> vals;
};

inline unsigned grid_for(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  return (unsigned)(g < 1 ? 1 : g);
}
