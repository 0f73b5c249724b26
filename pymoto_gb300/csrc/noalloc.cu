// pmg_dot_noalloc: the FP64-accumulated dot product for callers that cannot allocate device memory.
//
// pmg_dot needs a caller-provided scratch buffer for its per-CTA partial sums.  Some callers cannot
// provide one: a plugin running inside a host application that owns every device allocation (its own
// memory pool, no cudaMalloc allowed from third-party code), or code that runs where allocation is not
// permitted at all.  This variant keeps its scratch in a file-scope static device array instead, so the
// caller passes only the inputs and the output.
//
// Limits and sharing:
//  - The static scratch holds one partial sum per CTA, NOALLOC_MAX_CTAS of them; each CTA reduces
//    NOALLOC_CHUNK elements, so n may be at most NOALLOC_MAX_N = 4,194,304 elements.  Larger n is
//    rejected with PMG_BAD_ARG and a message in pmg_last_error().
//  - The array (about 32 KB) lives on every GPU that loads the library until the process exits.
//  - All calls on a device share the one array: calls that overlap on the GPU (different streams, or
//    different host threads without ordering between them) race and give wrong results.  Calls ordered on
//    one stream are safe.
//  - The first call on each device looks up the device address of the array (cudaGetSymbolAddress with
//    that device current).  Make that first call before any stream capture begins.
#include <mutex>

#include "common.cuh"

namespace pmg {
namespace {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_CHUNK = NOALLOC_THREADS * 4;
constexpr int NOALLOC_MAX_CTAS = 4096;
constexpr int64_t NOALLOC_MAX_N = (int64_t)NOALLOC_MAX_CTAS * NOALLOC_CHUNK;
constexpr int NOALLOC_MAX_CONTEXTS = 64;

struct NoAllocScratch {
  double partial[NOALLOC_MAX_CTAS];
  unsigned int ticket;
};

// The scratch: zero-initialised when the module loads, shared by every call on a device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// cached (context, address) pairs; the driver's cuCtxGetCurrent is reached through the runtime's entry-point
// query, so the library needs no link against libcuda
std::mutex g_noalloc_mutex;
void* g_noalloc_ctx[NOALLOC_MAX_CONTEXTS] = {};
NoAllocScratch* g_noalloc_addr[NOALLOC_MAX_CONTEXTS] = {};
int g_noalloc_count = 0;
typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn g_ctx_get_current = nullptr;

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ double na_block_sum(double v) {
  __shared__ double sh[NOALLOC_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = na_warp_sum(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (wid == 0) t = na_warp_sum(lane < NOALLOC_THREADS / 32 ? sh[lane] : 0.0);
  __syncthreads();
  return t;
}

// One CTA per NOALLOC_CHUNK elements; the last CTA to finish adds the partials in CTA order.
template <typename T>
__global__ void __launch_bounds__(NOALLOC_THREADS) dot_noalloc_kernel(int64_t n, const T* __restrict__ a,
                                                                      const T* __restrict__ b, double* out,
                                                                      NoAllocScratch* scr) {
  DotAcc<T> acc;
  const int64_t base = (int64_t)blockIdx.x * NOALLOC_CHUNK + threadIdx.x;
#pragma unroll
  for (int k = 0; k < NOALLOC_CHUNK / NOALLOC_THREADS; ++k) {
    const int64_t i = base + (int64_t)k * NOALLOC_THREADS;
    if (i < n) acc.add(a[i], b[i]);
  }
  double v = na_block_sum(acc.value());
  __shared__ bool last;
  if (threadIdx.x == 0) {
    scr->partial[blockIdx.x] = v;
    __threadfence();
    last = atomicAdd(&scr->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot = 0.0;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) tot += ((volatile double*)scr->partial)[c];
  tot = na_block_sum(tot);
  if (threadIdx.x == 0) {
    out[0] = tot;
    scr->ticket = 0u;
  }
}

// Device address of the static scratch in the current context, looked up once per context.
int scratch_address(NoAllocScratch** addr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);     // also makes the runtime bind its context to this thread
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_ctx_get_current == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == nullptr) {
      set_error("pmg_dot_noalloc: the driver's cuCtxGetCurrent is not available");
      return PMG_CUDA_ERR;
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  void* ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0 || ctx == nullptr) {
    set_error("pmg_dot_noalloc: no current CUDA context");
    return PMG_CUDA_ERR;
  }
  for (int i = 0; i < g_noalloc_count; ++i)
    if (g_noalloc_ctx[i] == ctx) {
      *addr = g_noalloc_addr[i];
      return PMG_OK;
    }
  if (g_noalloc_count >= NOALLOC_MAX_CONTEXTS) {
    set_error("pmg_dot_noalloc: more than 64 CUDA contexts");
    return PMG_BAD_ARG;
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) {
    set_error(e != cudaSuccess ? cudaGetErrorString(e) : "pmg_dot_noalloc: null scratch address");
    return PMG_CUDA_ERR;
  }
  g_noalloc_ctx[g_noalloc_count] = ctx;
  g_noalloc_addr[g_noalloc_count] = static_cast<NoAllocScratch*>(p);
  ++g_noalloc_count;
  *addr = g_noalloc_addr[g_noalloc_count - 1];
  return PMG_OK;
}

}  // namespace
}  // namespace pmg

using namespace pmg;

extern "C" {

int pmg_dot_noalloc(int dtype, int64_t n, const void* a, const void* b, double* out, void* stream) {
  if (n < 0 || !a || !b || !out || (dtype != PMG_F64 && dtype != PMG_F32)) {
    set_error("pmg_dot_noalloc: invalid argument");
    return PMG_BAD_ARG;
  }
  if (n > NOALLOC_MAX_N) {
    set_error("pmg_dot_noalloc: n exceeds the 4194304-element maximum of its static scratch; use pmg_dot");
    return PMG_BAD_ARG;
  }
  NoAllocScratch* scr = nullptr;
  int rc = scratch_address(&scr);
  if (rc != PMG_OK) return rc;
  cudaStream_t st = as_stream(stream);
  // the ticket must start at zero; the partials are written before they are read
  cudaError_t e = cudaMemsetAsync(&scr->ticket, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  int64_t nblk = (n + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK;
  if (nblk < 1) nblk = 1;
  if (dtype == PMG_F64)
    dot_noalloc_kernel<double><<<(unsigned)nblk, NOALLOC_THREADS, 0, st>>>(n, (const double*)a, (const double*)b, out,
                                                                           scr);
  else
    dot_noalloc_kernel<float><<<(unsigned)nblk, NOALLOC_THREADS, 0, st>>>(n, (const float*)a, (const float*)b, out,
                                                                          scr);
  return check_launch();
}

}  // extern "C"
