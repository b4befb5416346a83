// afp_matrix_vmult_noalloc: y = A x without any device allocation.
//
// afp_matrix_vmult stages x and y in two device buffers it allocates for the
// call.  Some callers cannot let a library allocate device memory when they
// call it: an application that reserved the whole device for its own memory
// arena up front, a process running under a hard device-memory cap, or a
// time-step loop that must not let the allocator's pool grow (or stall on
// it) inside the step.  This entry point stages x and y in one fixed array
// of static device storage instead (32 MiB per GPU).
//
// When the array is reserved: the library is built without relocatable
// device code, so this file is its own module, and CUDA loads modules lazily
// by default -- the array would otherwise appear on a GPU only when the
// module is first touched.  afp_context_create therefore looks the array up
// on its device (noalloc_reserve below), which loads the module and reserves
// the 32 MiB then; a caller that creates its context before handing the rest
// of the device to its own arena never sees the array appear later.  The
// array stays until the process exits.
//
// Limits and rules for the caller:
//  * matrices with more than AFP_NOALLOC_MAX_ENTRIES (2^21) rows or columns
//    are refused with AFP_ERR_UNSUPPORTED before anything is copied;
//  * every call, from any thread or context, uses the same array, so two
//    calls whose GPU work overlaps in time race and may return each other's
//    results -- serialise them;
//  * nothing in the array has to start at zero: x is copied over the first
//    half in full and every row of y is written by the product, so the
//    contents a previous call left behind are never read;
//  * the array's device address is looked up once per device ordinal (with
//    that device current) and kept for the life of the process; this
//    assumes the device's primary context lives as long, so do not call
//    cudaDeviceReset on a device this library has used.
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace {

constexpr int64_t kMaxEntries = AFP_NOALLOC_MAX_ENTRIES;
constexpr int kMaxDevices = 64;

// [0, kMaxEntries): x;  [kMaxEntries, 2 kMaxEntries): y.
static __device__ __align__(256) double g_vmult_stage[2 * kMaxEntries];

std::mutex g_stage_mu;
double* g_stage_addr[kMaxDevices] = {};

// Device address of g_vmult_stage on `device` (the current device).  In host
// code the symbol names a host-side placeholder, so the address must come
// from the runtime, once per device.
double* stage_on(int device) {
  AFP_REQUIRE(device >= 0 && device < kMaxDevices, AFP_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_stage_mu);
  if (g_stage_addr[device] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_vmult_stage);
    if (e != cudaSuccess)
      afp::fail(AFP_ERR_CUDA, std::string("afp_matrix_vmult_noalloc: cudaGetSymbolAddress failed: ") +
                                  cudaGetErrorString(e));
    g_stage_addr[device] = static_cast<double*>(p);
  }
  return g_stage_addr[device];
}

}  // namespace

namespace afp {
// Called by afp_context_create with `device` current: loads this module on
// the device and records the array's address, so the 32 MiB are reserved
// when the context is made, not inside a later afp_matrix_vmult_noalloc.
void noalloc_reserve(int device) { (void)stage_on(device); }
}  // namespace afp

extern "C" afp_status afp_matrix_vmult_noalloc(afp_matrix* a, const double* x, double* y) {
  using namespace afp;
  return guarded([&] {
    AFP_REQUIRE(a && x && y, AFP_ERR_INVALID, "null argument");
    const int64_t m = a->pat->m, n = a->pat->n;
    AFP_REQUIRE(m <= kMaxEntries && n <= kMaxEntries, AFP_ERR_UNSUPPORTED,
                "afp_matrix_vmult_noalloc: the matrix has more than AFP_NOALLOC_MAX_ENTRIES (2^21) rows or "
                "columns; use afp_matrix_vmult");
    afp_context* ctx = a->ctx;
    bind(ctx);
    double* stage = stage_on(ctx->device);
    double* sx = stage;
    double* sy = stage + kMaxEntries;
    copy(ctx, sx, x, sizeof(double) * n);
    csr_spmv(ctx, m, a->pat->rowptr.get(), a->pat->cols.get(), a->vals.get(), sx, sy);
    copy(ctx, y, sy, sizeof(double) * m);
    sync(ctx);
  });
}
