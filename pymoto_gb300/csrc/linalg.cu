// Reductions, CG vector updates, precision conversion and the FP64 banded Cholesky of the coarsest level.
#include "common.cuh"

namespace pmg {

// ------------------------------------------------------------------------------------------ reductions
// Deterministic single-launch reduction: every CTA writes its partial sums, the last CTA to finish
// (counted with an atomic ticket) adds the partials in CTA order and resets the ticket.
constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;
constexpr int RED_MAX_OUT = 2;

struct RedScratch {
  double partial[RED_MAX_OUT][RED_MAX_BLOCKS];
  unsigned int ticket;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of NOUT values; result valid in thread 0.
template <int NOUT>
__device__ __forceinline__ void block_sum(double (&v)[NOUT]) {
  __shared__ double sh[NOUT][RED_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NOUT; ++q) {
    v[q] = warp_sum(v[q]);
    if (lane == 0) sh[q][wid] = v[q];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NOUT; ++q) {
      double t = lane < (RED_THREADS / 32) ? sh[q][lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
}

// Writes the block partials and, in the last block, the totals to out[0..NOUT).
template <int NOUT>
__device__ __forceinline__ void finish_reduction(double (&v)[NOUT], RedScratch* scr, double* out) {
  block_sum<NOUT>(v);
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NOUT; ++q) scr->partial[q][blockIdx.x] = v[q];
    __threadfence();
    const unsigned t = atomicAdd(&scr->ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[NOUT];
#pragma unroll
  for (int q = 0; q < NOUT; ++q) acc[q] = 0.0;
  // fixed-order sum of the partials
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NOUT; ++q) acc[q] += ((volatile double*)scr->partial[q])[b];
  }
  block_sum<NOUT>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NOUT; ++q) out[q] = acc[q];
    scr->ticket = 0u;
  }
}

inline unsigned red_blocks(int64_t n) {
  int64_t b = (n + RED_THREADS * 4 - 1) / (RED_THREADS * 4);
  if (b < 1) b = 1;
  if (b > RED_MAX_BLOCKS) b = RED_MAX_BLOCKS;
  return (unsigned)b;
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) dot_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                                         double* out, RedScratch* scr) {
  double v[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[0] = fma((double)a[i], (double)b[i], v[0]);
  finish_reduction<1>(v, scr, out);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) dot2_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                                          const T* __restrict__ c, const T* __restrict__ d, double* out,
                                                          RedScratch* scr) {
  double v[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    v[0] = fma((double)a[i], (double)b[i], v[0]);
    v[1] = fma((double)c[i], (double)d[i], v[1]);
  }
  finish_reduction<2>(v, scr, out);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) cg_update_kernel(int64_t n, T* __restrict__ x, T* __restrict__ r,
                                                               const T* __restrict__ p, const T* __restrict__ q,
                                                               const double* num, const double* den, double* rr,
                                                               RedScratch* scr) {
  const double alpha = num[0] / den[0];
  const T a = (T)alpha;
  double v[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = x[i] + p[i] * a;
    const T ri = r[i] - q[i] * a;
    r[i] = ri;
    v[0] = fma((double)ri, (double)ri, v[0]);
  }
  finish_reduction<1>(v, scr, rr);
}

template <typename T>
__global__ void axpy_ratio_kernel(int64_t n, T* __restrict__ x, const T* __restrict__ p, const double* num,
                                  const double* den, double scale) {
  const T a = (T)(scale * (num[0] / den[0]));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] + p[i] * a;
}

template <typename T>
__global__ void xpby_ratio_kernel(int64_t n, T* __restrict__ p, const T* __restrict__ z, const double* num,
                                  const double* den) {
  const T beta = (T)(-(num[0] / den[0]));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + p[i] * beta;
}

template <typename T>
__global__ void scale_rsqrt_kernel(int64_t n, T* __restrict__ y, const T* __restrict__ x, const double* nrm2) {
  const double s = sqrt(nrm2[0]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (T)((double)x[i] / s);
}

template <typename T>
__global__ void scale_kernel(int64_t n, T* __restrict__ y, const T* __restrict__ x, T a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

template <typename T>
__global__ void mask_bc_kernel(int dim, int64_t nnodes, const uint8_t* __restrict__ m, int keep, const T* __restrict__ x,
                               T* __restrict__ y) {
  const int64_t n = nnodes * dim;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool bc = (m[i / dim] >> (i % dim)) & 1;
    y[i] = (bc == (keep != 0)) ? x[i] : T(0);
  }
}

template <typename S, typename D>
__global__ void convert_kernel(int64_t n, const S* __restrict__ x, D* __restrict__ y, double a) {
  if (a == 1.0) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      y[i] = (D)x[i];
  } else {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      y[i] = (D)(a * (double)x[i]);
  }
}

__global__ void add_f32_to_f64_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ d, double a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = fma(a, (double)d[i], x[i]);
}

template <typename T>
__global__ void diag_scale_kernel(int64_t n, const T* __restrict__ b, const T* __restrict__ diag, T w, T* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = w * (b[i] / diag[i]);
}

inline unsigned stream_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// ------------------------------------------------------------------------------------------ Cholesky
// Right-looking blocked Cholesky (lower, row-major, in place) with TB x TB tiles; tiles entirely outside
// the band stay zero and are skipped.
constexpr int TB = 32;

// Factor the diagonal tile kb in shared memory (one CTA of TB*TB/4 threads).
__global__ void chol_diag_kernel(int n, double* A, int kb, int* info) {
  __shared__ double T[TB][TB + 1];
  const int k0 = kb * TB;
  const int nb = min(TB, n - k0);
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    T[r][c] = (r < nb && c < nb) ? A[(int64_t)(k0 + r) * n + k0 + c] : (r == c ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    __shared__ double piv;
    if (threadIdx.x == 0) {
      double d = T[k][k];
      if (!(d > 0.0)) {
        if (*info == 0) *info = k0 + k + 1;
        d = 1.0;  // keep going with a unit pivot; the caller reports NOT_SPD
      }
      piv = sqrt(d);
      T[k][k] = piv;
    }
    __syncthreads();
    for (int r = k + 1 + threadIdx.x; r < nb; r += blockDim.x) T[r][k] /= piv;
    __syncthreads();
    for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
      const int r = e / TB, c = e % TB;
      if (r > k && c > k && c <= r && r < nb) T[r][c] -= T[r][k] * T[c][k];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    if (r < nb && c < nb) A[(int64_t)(k0 + r) * n + k0 + c] = c <= r ? T[r][c] : 0.0;
  }
}

// Panel: L[ib,kb] = A[ib,kb] L[kb,kb]^{-T}, one CTA (TB threads) per tile row ib > kb within the band.
__global__ void chol_panel_kernel(int n, double* A, int kb, int bw) {
  __shared__ double L[TB][TB + 1];
  const int k0 = kb * TB;
  const int nb = min(TB, n - k0);
  const int ib = kb + 1 + blockIdx.x;
  const int i0 = ib * TB;
  if (i0 >= n || i0 - (k0 + nb - 1) > bw) return;
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    L[r][c] = (r < nb && c < nb) ? A[(int64_t)(k0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  const int r = threadIdx.x;  // one row of the panel per thread
  const int row = i0 + r;
  if (r < TB && row < n) {
    double x[TB];
#pragma unroll
    for (int c = 0; c < TB; ++c) x[c] = c < nb ? A[(int64_t)row * n + k0 + c] : 0.0;
    // solve x L^T = a  (forward substitution over columns)
#pragma unroll
    for (int c = 0; c < TB; ++c) {
      if (c < nb) {
        double v = x[c];
#pragma unroll
        for (int q = 0; q < TB; ++q)
          if (q < c) v -= x[q] * L[c][q];
        x[c] = v / L[c][c];
      }
    }
#pragma unroll
    for (int c = 0; c < TB; ++c)
      if (c < nb) A[(int64_t)row * n + k0 + c] = x[c];
  }
}

// Trailing update A[ib,jb] -= L[ib,kb] L[jb,kb]^T for kb < jb <= ib within the band; one CTA per tile.
__global__ void chol_update_kernel(int n, double* A, int kb, int bw, int ntiles_band) {
  __shared__ double Li[TB][TB + 1];
  __shared__ double Lj[TB][TB + 1];
  const int k0 = kb * TB;
  const int nb = min(TB, n - k0);
  // tile enumeration: jb = kb+1+tj, ib = jb + ti, with ti, tj < ntiles_band
  const int tj = blockIdx.x % ntiles_band, ti = blockIdx.x / ntiles_band;
  const int jb = kb + 1 + tj, ib = jb + ti;
  const int i0 = ib * TB, j0 = jb * TB;
  if (i0 >= n || j0 >= n) return;
  if (i0 - (k0 + nb - 1) > bw || j0 - (k0 + nb - 1) > bw) return;  // L tiles are zero
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    Li[r][c] = (i0 + r < n && c < nb) ? A[(int64_t)(i0 + r) * n + k0 + c] : 0.0;
    Lj[r][c] = (j0 + r < n && c < nb) ? A[(int64_t)(j0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    const int row = i0 + r, col = j0 + c;
    if (row < n && col < n && col <= row) {
      double s = 0.0;
#pragma unroll 8
      for (int q = 0; q < TB; ++q) s = fma(Li[r][q], Lj[c][q], s);
      A[(int64_t)row * n + col] -= s;
    }
  }
}

// x = (L L^T)^{-1} b for a banded lower factor, one CTA: forward then backward substitution, with the
// band rows of each TB block updated in parallel.
template <typename T>
__global__ void __launch_bounds__(256) chol_solve_kernel(int n, const T* __restrict__ L, int bw, const T* __restrict__ b,
                                                        T* __restrict__ x) {
  // forward: y = L^{-1} b, stored in x
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
  __syncthreads();
  for (int k0 = 0; k0 < n; k0 += TB) {
    const int nb = min(TB, n - k0);
    if (threadIdx.x < 32) {
      // one warp solves the diagonal block sequentially
      for (int k = 0; k < nb; ++k) {
        T v = x[k0 + k];
        if (threadIdx.x == 0) {
          v = v / L[(int64_t)(k0 + k) * n + k0 + k];
          x[k0 + k] = v;
        }
        __syncwarp();
        v = x[k0 + k];
        const int r = k + 1 + threadIdx.x;
        if (r < nb) x[k0 + r] -= L[(int64_t)(k0 + r) * n + k0 + k] * v;
        __syncwarp();
      }
    }
    __syncthreads();
    // rows below the block within the band
    const int rend = min(n, k0 + nb + bw);
    for (int r = k0 + nb + threadIdx.x; r < rend; r += blockDim.x) {
      T s = T(0);
      for (int c = 0; c < nb; ++c) s += L[(int64_t)r * n + k0 + c] * x[k0 + c];
      x[r] -= s;
    }
    __syncthreads();
  }
  // backward: x = L^{-T} y
  const int nblk = (n + TB - 1) / TB;
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * TB;
    const int nb = min(TB, n - k0);
    if (threadIdx.x < 32) {
      for (int k = nb - 1; k >= 0; --k) {
        if (threadIdx.x == 0) x[k0 + k] = x[k0 + k] / L[(int64_t)(k0 + k) * n + k0 + k];
        __syncwarp();
        const T v = x[k0 + k];
        const int r = threadIdx.x;
        if (r < k) x[k0 + r] -= L[(int64_t)(k0 + k) * n + k0 + r] * v;
        __syncwarp();
      }
    }
    __syncthreads();
    // columns above the block within the band: x[c] -= sum_r L[r][c] x[r] for rows r in this block
    const int cbeg = max(0, k0 - bw);
    for (int c = cbeg + threadIdx.x; c < k0; c += blockDim.x) {
      T s = T(0);
      for (int r = 0; r < nb; ++r) s += L[(int64_t)(k0 + r) * n + c] * x[k0 + r];
      x[c] -= s;
    }
    __syncthreads();
  }
}

}  // namespace pmg

using namespace pmg;

extern "C" {

size_t pmg_reduce_scratch_bytes(void) { return sizeof(RedScratch); }

int pmg_dot(int dtype, int64_t n, const void* a, const void* b, double* out, void* scratch, void* stream) {
  if (n < 0 || !a || !b || !out || !scratch || (dtype != PMG_F64 && dtype != PMG_F32)) return PMG_BAD_ARG;
  const unsigned g = red_blocks(n);
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    dot_kernel<double><<<g, RED_THREADS, 0, st>>>(n, (const double*)a, (const double*)b, out, (RedScratch*)scratch);
  else
    dot_kernel<float><<<g, RED_THREADS, 0, st>>>(n, (const float*)a, (const float*)b, out, (RedScratch*)scratch);
  return check_launch();
}

int pmg_dot2(int dtype, int64_t n, const void* a, const void* b, const void* c, const void* d, double* out,
             void* scratch, void* stream) {
  if (n < 0 || !a || !b || !c || !d || !out || !scratch || (dtype != PMG_F64 && dtype != PMG_F32)) return PMG_BAD_ARG;
  const unsigned g = red_blocks(n);
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    dot2_kernel<double><<<g, RED_THREADS, 0, st>>>(n, (const double*)a, (const double*)b, (const double*)c,
                                                   (const double*)d, out, (RedScratch*)scratch);
  else
    dot2_kernel<float><<<g, RED_THREADS, 0, st>>>(n, (const float*)a, (const float*)b, (const float*)c,
                                                  (const float*)d, out, (RedScratch*)scratch);
  return check_launch();
}

int pmg_cg_update(int dtype, int64_t n, void* x, void* r, const void* p, const void* q, const double* num,
                  const double* den, double* rr_out, void* scratch, void* stream) {
  if (n < 0 || !x || !r || !p || !q || !num || !den || !rr_out || !scratch) return PMG_BAD_ARG;
  const unsigned g = red_blocks(n);
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    cg_update_kernel<double><<<g, RED_THREADS, 0, st>>>(n, (double*)x, (double*)r, (const double*)p, (const double*)q,
                                                        num, den, rr_out, (RedScratch*)scratch);
  else if (dtype == PMG_F32)
    cg_update_kernel<float><<<g, RED_THREADS, 0, st>>>(n, (float*)x, (float*)r, (const float*)p, (const float*)q, num,
                                                       den, rr_out, (RedScratch*)scratch);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_axpy_ratio(int dtype, int64_t n, void* x, const void* p, const double* num, const double* den, double scale,
                   void* stream) {
  if (n < 0 || !x || !p || !num || !den) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    axpy_ratio_kernel<double><<<stream_blocks(n), 256, 0, st>>>(n, (double*)x, (const double*)p, num, den, scale);
  else if (dtype == PMG_F32)
    axpy_ratio_kernel<float><<<stream_blocks(n), 256, 0, st>>>(n, (float*)x, (const float*)p, num, den, scale);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_xpby_ratio(int dtype, int64_t n, void* p, const void* z, const double* num, const double* den, void* stream) {
  if (n < 0 || !p || !z || !num || !den) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    xpby_ratio_kernel<double><<<stream_blocks(n), 256, 0, st>>>(n, (double*)p, (const double*)z, num, den);
  else if (dtype == PMG_F32)
    xpby_ratio_kernel<float><<<stream_blocks(n), 256, 0, st>>>(n, (float*)p, (const float*)z, num, den);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_scale_rsqrt(int dtype, int64_t n, void* y, const void* x, const double* nrm2, void* stream) {
  if (n < 0 || !x || !y || !nrm2) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    scale_rsqrt_kernel<double><<<stream_blocks(n), 256, 0, st>>>(n, (double*)y, (const double*)x, nrm2);
  else if (dtype == PMG_F32)
    scale_rsqrt_kernel<float><<<stream_blocks(n), 256, 0, st>>>(n, (float*)y, (const float*)x, nrm2);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_scale(int dtype, int64_t n, void* y, const void* x, double a, void* stream) {
  if (n < 0 || !x || !y) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    scale_kernel<double><<<stream_blocks(n), 256, 0, st>>>(n, (double*)y, (const double*)x, a);
  else if (dtype == PMG_F32)
    scale_kernel<float><<<stream_blocks(n), 256, 0, st>>>(n, (float*)y, (const float*)x, (float)a);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_mask_bc(int dtype, int dim, int64_t nnodes, const uint8_t* bcmask, int keep_bc, const void* x, void* y,
                void* stream) {
  if (nnodes < 0 || (dim != 2 && dim != 3) || !bcmask || !x || !y) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const int64_t n = nnodes * dim;
  if (dtype == PMG_F64)
    mask_bc_kernel<double><<<stream_blocks(n), 256, 0, st>>>(dim, nnodes, bcmask, keep_bc, (const double*)x, (double*)y);
  else if (dtype == PMG_F32)
    mask_bc_kernel<float><<<stream_blocks(n), 256, 0, st>>>(dim, nnodes, bcmask, keep_bc, (const float*)x, (float*)y);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_convert(int src_dtype, int dst_dtype, int64_t n, const void* x, void* y, double a, void* stream) {
  if (n < 0 || !x || !y) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const unsigned g = stream_blocks(n);
  if (src_dtype == PMG_F64 && dst_dtype == PMG_F32)
    convert_kernel<double, float><<<g, 256, 0, st>>>(n, (const double*)x, (float*)y, a);
  else if (src_dtype == PMG_F32 && dst_dtype == PMG_F64)
    convert_kernel<float, double><<<g, 256, 0, st>>>(n, (const float*)x, (double*)y, a);
  else if (src_dtype == PMG_F64 && dst_dtype == PMG_F64)
    convert_kernel<double, double><<<g, 256, 0, st>>>(n, (const double*)x, (double*)y, a);
  else if (src_dtype == PMG_F32 && dst_dtype == PMG_F32)
    convert_kernel<float, float><<<g, 256, 0, st>>>(n, (const float*)x, (float*)y, a);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_add_f32_to_f64(int64_t n, double* x, const float* d, double a, void* stream) {
  if (n < 0 || !x || !d) return PMG_BAD_ARG;
  add_f32_to_f64_kernel<<<stream_blocks(n), 256, 0, as_stream(stream)>>>(n, x, d, a);
  return check_launch();
}

int pmg_diag_scale(int dtype, int64_t n, const void* b, const void* diag, double w, void* y, void* stream) {
  if (n < 0 || !b || !diag || !y) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    diag_scale_kernel<double><<<stream_blocks(n), 256, 0, st>>>(n, (const double*)b, (const double*)diag, w, (double*)y);
  else if (dtype == PMG_F32)
    diag_scale_kernel<float><<<stream_blocks(n), 256, 0, st>>>(n, (const float*)b, (const float*)diag, (float)w, (float*)y);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_cholesky_factor(int n, double* A, int bw, int* info, void* stream) {
  if (n <= 0 || !A || !info || bw < 0) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int), st);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  const int nblk = (n + TB - 1) / TB;
  const int band_tiles = min(nblk, bw / TB + 2);
  for (int kb = 0; kb < nblk; ++kb) {
    chol_diag_kernel<<<1, 256, 0, st>>>(n, A, kb, info);
    const int rem = nblk - kb - 1;
    if (rem <= 0) break;
    const int pt = min(rem, band_tiles);
    chol_panel_kernel<<<pt, TB, 0, st>>>(n, A, kb, bw);
    chol_update_kernel<<<pt * pt, 256, 0, st>>>(n, A, kb, bw, pt);
    const int rc = check_launch();
    if (rc != PMG_OK) return rc;
  }
  return check_launch();
}

int pmg_cholesky_solve(int dtype, int n, const void* L, int bw, const void* b, void* x, void* stream) {
  if (n <= 0 || !L || !b || !x || bw < 0 || b == x) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    chol_solve_kernel<double><<<1, 256, 0, st>>>(n, (const double*)L, bw, (const double*)b, (double*)x);
  else if (dtype == PMG_F32)
    chol_solve_kernel<float><<<1, 256, 0, st>>>(n, (const float*)L, bw, (const float*)b, (float*)x);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

}  // extern "C"
