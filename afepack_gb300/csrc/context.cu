// Context, errors, copies, device scan and the matrix handle of the C ABI.
#include <cstring>

#include "common.cuh"
#include "kernels.cuh"

namespace afp {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

void bind(const afp_context* ctx) { AFP_CUDA(cudaSetDevice(ctx->device)); }

void copy(const afp_context* ctx, void* dst, const void* src, size_t bytes) {
  if (bytes) AFP_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
}

void sync(const afp_context* ctx) { AFP_CUDA(cudaStreamSynchronize(ctx->stream)); }

void check_launch(const afp_context* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fail(AFP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  const_cast<afp_context*>(ctx)->launches.n++;
}

// ------------------------------------------------------------------ scan
// Three-phase exclusive scan: per-tile totals, a sequential scan of the tile
// totals by one block, then per-tile scans offset by their tile's prefix.
static constexpr int SCAN_THREADS = 256;
static constexpr int SCAN_ITEMS = 8;
static constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t s = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SCAN_THREADS / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  int64_t before = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
  *total = warp_sums[SCAN_THREADS / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void k_tile_totals(const int* __restrict__ in, int64_t n, int64_t* __restrict__ tiles) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int64_t i = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  int64_t total;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) tiles[blockIdx.x] = total;
}

__global__ void k_scan_tiles(int64_t* tiles, int64_t ntiles, int64_t* grand) {
  int64_t carry = 0;
  for (int64_t base = 0; base < ntiles; base += SCAN_THREADS) {
    int64_t i = base + threadIdx.x;
    int64_t v = i < ntiles ? tiles[i] : 0;
    int64_t total;
    int64_t ex = block_exclusive_scan(v, &total);
    if (i < ntiles) tiles[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *grand = carry;
}

__global__ void k_tile_scan(const int* __restrict__ in, int64_t n, const int64_t* __restrict__ tiles,
                            int* __restrict__ out, const int64_t* grand) {
  __shared__ int64_t carry_s;
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  if (threadIdx.x == 0) carry_s = tiles[blockIdx.x];
  __syncthreads();
  // items of a thread are contiguous so the scan is in index order
  int64_t vals[SCAN_ITEMS];
  int64_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    vals[k] = i < n ? in[i] : 0;
    s += vals[k];
  }
  int64_t total;
  int64_t run = carry_s + block_exclusive_scan(s, &total);
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    if (i < n) out[i] = (int)run;
    run += vals[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = (int)*grand;
}

int64_t exclusive_scan(const afp_context* ctx, const int* counts, int* out, int64_t n) {
  int64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles < 1) ntiles = 1;
  DevBuf<int64_t> tiles(ctx, (size_t)ntiles + 1);
  k_tile_totals<<<(unsigned)ntiles, SCAN_THREADS, 0, ctx->stream>>>(counts, n, tiles.get());
  check_launch(ctx, "scan totals");
  k_scan_tiles<<<1, SCAN_THREADS, 0, ctx->stream>>>(tiles.get(), ntiles, tiles.get() + ntiles);
  check_launch(ctx, "scan tiles");
  k_tile_scan<<<(unsigned)ntiles, SCAN_THREADS, 0, ctx->stream>>>(counts, n, tiles.get(), out,
                                                                     tiles.get() + ntiles);
  check_launch(ctx, "scan");
  int64_t total = 0;
  copy(ctx, &total, tiles.get() + ntiles, sizeof(int64_t));
  sync(ctx);
  AFP_REQUIRE(total < (int64_t)INT32_MAX, AFP_ERR_UNSUPPORTED,
              "more than 2^31-1 stored entries in one matrix");
  return total;
}

}  // namespace afp

using namespace afp;

// ====================================================================== C ABI
extern "C" {

int afp_version(void) { return AFP_VERSION; }

const char* afp_status_string(afp_status s) {
  switch (s) {
    case AFP_OK: return "ok";
    case AFP_ERR_INVALID: return "invalid argument";
    case AFP_ERR_CUDA: return "CUDA error";
    case AFP_ERR_NO_DEVICE: return "no usable GPU";
    case AFP_ERR_OUT_OF_MEMORY: return "out of memory";
    case AFP_ERR_NOT_CONVERGED: return "not converged";
    case AFP_ERR_BREAKDOWN: return "breakdown (NaN/Inf or zero denominator)";
    case AFP_ERR_SINGULAR: return "singular coarsest matrix";
    case AFP_ERR_TIMEOUT: return "timeout";
    case AFP_ERR_UNSUPPORTED: return "unsupported input";
    case AFP_ERR_CAPACITY: return "capacity exceeded";
  }
  return "unknown status";
}

const char* afp_last_error(void) { return g_last_error.c_str(); }

afp_status afp_context_create(int device, afp_context** out) {
  return guarded([&] {
    AFP_REQUIRE(out != nullptr, AFP_ERR_INVALID, "out is NULL");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
      fail(AFP_ERR_NO_DEVICE, "no CUDA device visible");
    AFP_REQUIRE(device >= 0 && device < count, AFP_ERR_INVALID, "device index out of range");
    AFP_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    AFP_CUDA(cudaGetDeviceProperties(&prop, device));
    AFP_REQUIRE(prop.major == 10 && prop.minor == 3, AFP_ERR_NO_DEVICE,
                std::string("kernels are built for sm_103a; device is sm_") + std::to_string(prop.major) +
                    std::to_string(prop.minor));
    auto ctx = std::make_unique<afp_context>();
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    AFP_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    // keep freed blocks in the stream-ordered pool instead of returning them
    cudaMemPool_t pool;
    AFP_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t threshold = UINT64_MAX;
    AFP_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
    AFP_CUDA(cudaMalloc(&ctx->d_scalars, 64 * sizeof(double)));
    AFP_CUDA(cudaMalloc(&ctx->d_partials, 1024 * sizeof(double)));
    AFP_CUDA(cudaMalloc(&ctx->d_retire, 16 * sizeof(unsigned)));
    AFP_CUDA(cudaMemset(ctx->d_retire, 0, 16 * sizeof(unsigned)));
    AFP_CUDA(cudaMallocHost(&ctx->h_scalars, 64 * sizeof(double)));
    noalloc_reserve(device);
    *out = ctx.release();
  });
}

afp_status afp_context_destroy(afp_context* ctx) {
  return guarded([&] {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_scalars);
    cudaFree(ctx->d_partials);
    cudaFree(ctx->d_retire);
    cudaFreeHost(ctx->h_scalars);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
  });
}

afp_status afp_context_synchronize(afp_context* ctx) {
  return guarded([&] {
    AFP_REQUIRE(ctx, AFP_ERR_INVALID, "null context");
    bind(ctx);
    sync(ctx);
  });
}

afp_status afp_context_stream(const afp_context* ctx, void** stream) {
  return guarded([&] {
    AFP_REQUIRE(ctx && stream, AFP_ERR_INVALID, "null argument");
    *stream = (void*)ctx->stream;
  });
}

afp_status afp_context_launch_count(const afp_context* ctx, int64_t* count) {
  return guarded([&] {
    AFP_REQUIRE(ctx && count, AFP_ERR_INVALID, "null argument");
    *count = ctx->launches.n;
  });
}

afp_status afp_matrix_create_csr(afp_context* ctx, int64_t m, int64_t n, int64_t nnz, const int32_t* rowptr,
                                 const int32_t* cols, const double* vals, afp_matrix** out) {
  return guarded([&] {
    AFP_REQUIRE(ctx && rowptr && cols && vals && out, AFP_ERR_INVALID, "null argument");
    AFP_REQUIRE(m > 0 && n > 0 && nnz >= m && nnz < INT32_MAX, AFP_ERR_INVALID, "bad matrix sizes");
    bind(ctx);
    auto A = std::make_unique<afp_matrix>();
    A->ctx = ctx;
    A->pat = std::make_shared<Pattern>();
    A->pat->m = m;
    A->pat->n = n;
    A->pat->nnz = nnz;
    A->pat->rowptr.alloc(ctx, m + 1);
    A->pat->cols.alloc(ctx, nnz);
    A->vals.alloc(ctx, nnz);
    A->pat->rowptr.upload(rowptr, m + 1);
    A->pat->cols.upload(cols, nnz);
    A->vals.upload(vals, nnz);
    sync(ctx);
    *out = A.release();
  });
}

afp_status afp_matrix_info(const afp_matrix* a, int64_t* m, int64_t* n, int64_t* nnz) {
  return guarded([&] {
    AFP_REQUIRE(a, AFP_ERR_INVALID, "null matrix");
    if (m) *m = a->pat->m;
    if (n) *n = a->pat->n;
    if (nnz) *nnz = a->pat->nnz;
  });
}

afp_status afp_matrix_set_values(afp_matrix* a, const double* vals) {
  return guarded([&] {
    AFP_REQUIRE(a && vals, AFP_ERR_INVALID, "null argument");
    bind(a->ctx);
    a->vals.upload(vals, a->pat->nnz);
    sync(a->ctx);
  });
}

afp_status afp_matrix_download(const afp_matrix* a, int32_t* rowptr, int32_t* cols, double* vals) {
  return guarded([&] {
    AFP_REQUIRE(a, AFP_ERR_INVALID, "null matrix");
    bind(a->ctx);
    if (rowptr) a->pat->rowptr.download(rowptr, a->pat->m + 1);
    if (cols) a->pat->cols.download(cols, a->pat->nnz);
    if (vals) a->vals.download(vals, a->pat->nnz);
    sync(a->ctx);
  });
}

afp_status afp_matrix_vmult(afp_matrix* a, const double* x, double* y) {
  return guarded([&] {
    AFP_REQUIRE(a && x && y, AFP_ERR_INVALID, "null argument");
    afp_context* ctx = a->ctx;
    bind(ctx);
    DevBuf<double> dx(ctx, a->pat->n), dy(ctx, a->pat->m);
    dx.upload(x, a->pat->n);
    csr_spmv(ctx, a->pat->m, a->pat->rowptr.get(), a->pat->cols.get(), a->vals.get(), dx.get(), dy.get());
    dy.download(y, a->pat->m);
    sync(ctx);
  });
}

afp_status afp_matrix_destroy(afp_matrix* a) {
  return guarded([&] {
    if (!a) return;
    bind(a->ctx);
    sync(a->ctx);
    delete a;
  });
}

void afp_host_free(void* p) { std::free(p); }

}  // extern "C"
