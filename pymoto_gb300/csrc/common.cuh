// Shared definitions of the pymoto_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "../../include/pymoto_gb300.h"

namespace pmg {

// Structured voxel grid given by its element counts; nz == 0 is the 2D grid.
struct Grid {
  int nx, ny, nz;
  __host__ __device__ int dim() const { return nz == 0 ? 2 : 3; }
  __host__ __device__ int nnx() const { return nx + 1; }
  __host__ __device__ int nny() const { return ny + 1; }
  __host__ __device__ int nnz() const { return nz + 1; }
  __host__ __device__ int ez() const { return nz == 0 ? 1 : nz; }  // element layers
  __host__ __device__ int64_t nel() const { return (int64_t)nx * ny * ez(); }
  __host__ __device__ int64_t nnodes() const { return (int64_t)(nx + 1) * (ny + 1) * (nz + 1); }
  __host__ __device__ Grid coarse() const { return Grid{nx / 2, ny / 2, nz / 2}; }
};

template <int DIM>
struct Traits {
  static constexpr int NN = 1 << DIM;         // nodes per element
  static constexpr int NDE = NN * DIM;        // dofs per element
  static constexpr int NOFF = DIM == 3 ? 27 : 9;  // node-stencil offsets
  // Node stencils of the (symmetric) operators are stored half: the centre block and the blocks of the
  // forward offsets o > CENTER, o = (dz+1)*9 + (dy+1)*3 + (dx+1), as S[(h*DIM + d)*DIM + c][node] with
  // h = o - CENTER.  The block of a backward offset o < CENTER at node n is the transpose of the stored block
  // of the neighbour m = n + off(o) at offset NOFF-1-o.
  static constexpr int CENTER = NOFF / 2;          // 13 (3D), 4 (2D)
  static constexpr int NH = NOFF - CENTER;         // stored offsets per node: 14, 5
  static constexpr int NSB = NH * DIM * DIM;       // stored stencil values per node: 126, 20
};

// (dx, dy, dz) of node-stencil offset o
template <int DIM>
__host__ __device__ __forceinline__ void stencil_offset(int o, int& dx, int& dy, int& dz) {
  dx = o % 3 - 1;
  dy = (o / 3) % 3 - 1;
  dz = DIM == 3 ? o / 9 - 1 : 0;
}

// Element matrix passed by value in the kernel parameter space (constant bank): all threads of a warp
// read the same entry at the same time, so the FMAs take it as a uniform operand.
template <typename T, int NDE>
struct ElemMat {
  T v[NDE * NDE];
};

// Thread-local error of the last failing call.
void set_error(const char* msg);
const char* last_error();

inline int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return PMG_OK;
}

inline bool grid_ok(int nx, int ny, int nz) {
  return nx > 0 && ny > 0 && nz >= 0 && (int64_t)(nx + 1) * (ny + 1) * (nz + 1) < (int64_t(1) << 31);
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// Multiprocessor count of the current device (cached per device).
inline int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  if (!cache[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = v > 0 ? v : 1;
  }
  return cache[dev];
}

template <typename T, int NDE>
inline ElemMat<T, NDE> make_elem_mat(const double* K0) {
  ElemMat<T, NDE> m;
  for (int i = 0; i < NDE * NDE; ++i) m.v[i] = (T)K0[i];
  return m;
}

// Node coordinates from a linear node index.  Node and element counts are below 2^31 (checked by every
// entry point), so the index arithmetic is 32-bit: 64-bit division costs hundreds of instructions.
__device__ __forceinline__ void node_ijk(const Grid& g, int64_t n64, int& i, int& j, int& k) {
  const unsigned n = (unsigned)n64, nnx = (unsigned)(g.nx + 1), nny = (unsigned)(g.ny + 1);
  const unsigned t = n / nnx;
  i = (int)(n - t * nnx);
  k = (int)(t / nny);
  j = (int)(t - (unsigned)k * nny);
}

__device__ __forceinline__ int64_t node_id(const Grid& g, int i, int j, int k) {
  return (int64_t)((k * (g.ny + 1) + j) * (g.nx + 1) + i);
}

__device__ __forceinline__ int64_t elem_id(const Grid& g, int i, int j, int k) {
  return (int64_t)((k * g.ny + j) * g.nx + i);
}

// Operands of the fused Chebyshev smoothing step (operator apply mode 3): with r = b - A u,
// d <- a_j d + c_j r / diag (a_0 = 0: d not read at step 0), y = u + d; coef[2j], coef[2j+1] = a_j, c_j.
template <typename T>
struct ChebArgs {
  T* d;
  const double* coef;
  int step;
};
constexpr int PMG_APPLY_CHEB = 3;

// Dot-product accumulators.  FP64 data: one FP64 FMA per element.  FP32 data: no FP64 arithmetic per element
// (GB300 runs FP64 at 1/64 of the FP32 rate); the product is split exactly into p + e with an FMA and added
// to an unevaluated sum s + c by Knuth's TwoSum (Ogita, Rump, Oishi, "Accurate sum and dot product", SIAM J.
// Sci. Comput. 26 (2005), Dot2), which is as accurate as FP64 accumulation of the exact products.  The
// explicitly rounded intrinsics keep the compiler from contracting the error terms into FMAs.
template <typename T>
struct DotAcc;

template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};

template <>
struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = fmaf(a, b, -p);                  // a b - p, exact
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));   // s + p - t, exact
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// 3D FP32 operator apply on the tensor cores (ebe_tc.cu: tcgen05, accumulators in tensor memory).
int ebe_apply_tc_f32(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                     const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                     const float* cdiag, cudaStream_t st);
// The same on the CUDA cores (ebe_fma.cu: one thread per node column, FP32 FMAs).
int ebe_apply_fma_f32(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                      const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                      const float* cdiag, cudaStream_t st);
// The implementation selected by pmg_set_operator_kernel.
int ebe_apply_f32_3d(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                     const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                     const float* cdiag, cudaStream_t st);


}  // namespace pmg
