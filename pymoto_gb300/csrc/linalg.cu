// Reductions, CG vector updates, precision conversion and the FP64 banded Cholesky of the coarsest level.
#include <algorithm>

#include "common.cuh"

namespace pmg {

// ------------------------------------------------------------------------------------------ reductions
// Deterministic single-launch reduction: every CTA writes its partial sums, the last CTA to finish
// (counted with an atomic ticket) adds the partials in CTA order and resets the ticket.
constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 2048;
constexpr int RED_MAX_OUT = 2;
constexpr int ILP = 4;  // elements per thread and pass in the streaming kernels

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

// Four CTAs per SM at most (grid-stride): each thread reduces ~10 elements of a 1.6M vector in registers, so
// the FP64 block and grid sums (a warp-wide FP64 add costs 16 cycles of an SM on GB300) stay a small part.
inline unsigned red_blocks(int64_t n) {
  int64_t b = (n + RED_THREADS * ILP - 1) / (RED_THREADS * ILP);
  const int64_t cap = std::min<int64_t>(RED_MAX_BLOCKS, 4 * (int64_t)sm_count());
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// Scalar num/den (times scale) computed once per CTA: an FP64 division per thread is expensive on GB300.
// A zero denominator gives a zero ratio (no update) instead of inf/nan.
__device__ __forceinline__ double cta_ratio(const double* num, const double* den, double scale) {
  __shared__ double s_ratio;
  if (threadIdx.x == 0) s_ratio = den[0] != 0.0 ? scale * (num[0] / den[0]) : 0.0;
  __syncthreads();
  return s_ratio;
}

// Element loops of the streaming kernels: each thread takes ILP elements per pass (strided by the CTA width,
// so every load instruction of a warp is coalesced) and keeps their loads in flight together.
#define PMG_ILP_LOOP(n, BODY)                                                                               \
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x * ILP + threadIdx.x; base < (n);                     \
       base += (int64_t)gridDim.x * blockDim.x * ILP) {                                                     \
    _Pragma("unroll") for (int k_ = 0; k_ < ILP; ++k_) {                                                    \
      const int64_t i = base + (int64_t)k_ * blockDim.x;                                                    \
      if (i < (n)) { BODY; }                                                                                \
    }                                                                                                       \
  }

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) dot_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                                         double* out, RedScratch* scr) {
  DotAcc<T> acc;
  PMG_ILP_LOOP(n, acc.add(a[i], b[i]))
  double v[1] = {acc.value()};
  finish_reduction<1>(v, scr, out);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) dot2_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b,
                                                          const T* __restrict__ c, const T* __restrict__ d, double* out,
                                                          RedScratch* scr) {
  DotAcc<T> acc0, acc1;
  PMG_ILP_LOOP(n, acc0.add(a[i], b[i]); acc1.add(c[i], d[i]))
  double v[2] = {acc0.value(), acc1.value()};
  finish_reduction<2>(v, scr, out);
}

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) cg_update_kernel(int64_t n, T* __restrict__ x, T* __restrict__ r,
                                                               const T* __restrict__ p, const T* __restrict__ q,
                                                               const double* num, const double* den, double* rr,
                                                               RedScratch* scr) {
  const T a = (T)cta_ratio(num, den, 1.0);
  DotAcc<T> acc;
  PMG_ILP_LOOP(n, x[i] = x[i] + p[i] * a; const T ri = r[i] - q[i] * a; r[i] = ri; acc.add(ri, ri))
  double v[1] = {acc.value()};
  finish_reduction<1>(v, scr, rr);
}

template <typename T>
__global__ void axpy_ratio_kernel(int64_t n, T* __restrict__ x, const T* __restrict__ p, const double* num,
                                  const double* den, double scale) {
  const T a = (T)cta_ratio(num, den, scale);
  PMG_ILP_LOOP(n, x[i] = x[i] + p[i] * a)
}

template <typename T>
__global__ void xpby_ratio_kernel(int64_t n, T* __restrict__ p, const T* __restrict__ z, const double* num,
                                  const double* den) {
  const T beta = (T)cta_ratio(num, den, -1.0);
  PMG_ILP_LOOP(n, p[i] = z[i] + p[i] * beta)
}

template <typename T>
__global__ void scale_rsqrt_kernel(int64_t n, T* __restrict__ y, const T* __restrict__ x, const double* nrm2) {
  __shared__ double s_inv;
  if (threadIdx.x == 0) s_inv = nrm2[0] > 0.0 ? 1.0 / sqrt(nrm2[0]) : 0.0;
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, step = (int64_t)gridDim.x * blockDim.x;
  if (sizeof(T) == 4 && s_inv < 1e37) {
    // FP32 data with a representable scale: rounded once, no FP64 arithmetic per element
    const T s = (T)s_inv;
    for (int64_t i = i0; i < n; i += step) y[i] = x[i] * s;
  } else {
    const double s = s_inv;
    for (int64_t i = i0; i < n; i += step) y[i] = (T)((double)x[i] * s);
  }
}

template <typename T>
__global__ void scale_kernel(int64_t n, T* __restrict__ y, const T* __restrict__ x, T a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

// One thread per node (the mask byte is read once, no index division).
template <typename T, int DIM>
__global__ void mask_bc_kernel(int64_t nnodes, const uint8_t* __restrict__ m, int keep, const T* __restrict__ x,
                               T* __restrict__ y) {
  for (int64_t nd = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; nd < nnodes; nd += (int64_t)gridDim.x * blockDim.x) {
    const unsigned mm = m[nd];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const bool bc = (mm >> d) & 1u;
      y[nd * DIM + d] = (bc == (keep != 0)) ? x[nd * DIM + d] : T(0);
    }
  }
}

// Dirichlet split of a right-hand side in one pass: direct = rhs / bcdiag on constrained dofs (0 elsewhere),
// free = rhs on free dofs (0 on constrained ones).
template <typename T, int DIM>
__global__ void split_bc_kernel(int64_t nnodes, const uint8_t* __restrict__ m, T bcdiag, const T* __restrict__ rhs,
                                T* __restrict__ direct, T* __restrict__ free_part, const T* __restrict__ cdiag) {
  for (int64_t nd = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; nd < nnodes; nd += (int64_t)gridDim.x * blockDim.x) {
    const unsigned mm = m[nd];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const T v = rhs[nd * DIM + d];
      const bool bc = (mm >> d) & 1u;
      // a Dirichlet row holds bcdiag (+ the constant diagonal term) only
      direct[nd * DIM + d] = bc ? v / (bcdiag + (cdiag ? cdiag[nd * DIM + d] : T(0))) : T(0);
      free_part[nd * DIM + d] = bc ? T(0) : v;
    }
  }
}

template <typename S, typename D>
__global__ void convert_kernel(int64_t n, const S* __restrict__ x, D* __restrict__ y, double a) {
  if (a == 1.0) {
    PMG_ILP_LOOP(n, y[i] = (D)x[i])
  } else {
    PMG_ILP_LOOP(n, y[i] = (D)(a * (double)x[i]))
  }
}

// y = x * sqrt(s[0]) or x / sqrt(s[0]) (inverse != 0): the scale comes from device memory
template <typename S, typename D>
__global__ void convert_dscale_kernel(int64_t n, const S* __restrict__ x, D* __restrict__ y, const double* s,
                                      int inverse) {
  __shared__ double sc;
  if (threadIdx.x == 0) {
    const double v = s[0];
    sc = inverse ? (v > 0.0 ? 1.0 / sqrt(v) : 0.0) : sqrt(v > 0.0 ? v : 0.0);
  }
  __syncthreads();
  const double a = sc;
  PMG_ILP_LOOP(n, y[i] = (D)(a * (double)x[i]))
}

__global__ void add_f32_to_f64_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ d, double a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = fma(a, (double)d[i], x[i]);
}

template <typename T>
__global__ void diag_scale_kernel(int64_t n, const T* __restrict__ b, const T* __restrict__ diag, T w, T* __restrict__ y) {
  PMG_ILP_LOOP(n, y[i] = w * (b[i] / diag[i]))
}

// Chebyshev smoothing (polynomial in D^-1 A on [lmax/ratio, lmax]; Saad, Iterative Methods for Sparse
// Linear Systems, 2nd ed., Alg. 12.1): step j updates d <- a_j d + c_j D^-1 r, x <- x + d, with
// a_0 = 0, c_0 = 1/theta, a_j = rho_j rho_{j-1}, c_j = 2 rho_j / delta, rho_0 = 1/sigma,
// rho_j = 1/(2 sigma - rho_{j-1}), theta = (lmax + lmin)/2, delta = (lmax - lmin)/2, sigma = theta/delta.
__global__ void cheb_coeffs_kernel(const double* __restrict__ lmax_dev, double lmax_host, double ratio, int degree,
                                   double* __restrict__ coef) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double hi = lmax_dev ? *lmax_dev : lmax_host;
  if (!(hi > 0.0)) hi = 1.0;
  const double lo = hi / ratio;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
  double rho = 1.0 / sigma;
  coef[0] = 0.0;
  coef[1] = 1.0 / theta;
  for (int j = 1; j < degree; ++j) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    coef[2 * j] = rn * rho;
    coef[2 * j + 1] = 2.0 * rn / delta;
    rho = rn;
  }
}

// d = a_j d + c_j r / diag; x = x + d (init != 0: the first step from x = 0, d = c_0 r / diag, x = d)
template <typename T>
__global__ void cheb_step_kernel(int64_t n, const T* __restrict__ r, const T* __restrict__ diag, T* __restrict__ d,
                                 T* __restrict__ x, const double* __restrict__ coef, int step, int init) {
  const T a = (T)coef[2 * step], c = (T)coef[2 * step + 1];
  if (init) {
    PMG_ILP_LOOP(n, { const T v = c * (r[i] / diag[i]); d[i] = v; x[i] = v; })
  } else if (step == 0) {   // a_0 = 0: d is not read
    PMG_ILP_LOOP(n, { const T v = c * (r[i] / diag[i]); d[i] = v; x[i] += v; })
  } else {
    PMG_ILP_LOOP(n, { const T v = a * d[i] + c * (r[i] / diag[i]); d[i] = v; x[i] += v; })
  }
}

inline unsigned stream_blocks(int64_t n) {
  int64_t b = (n + 256 * ILP - 1) / (256 * ILP);
  if (b > 65535) b = 65535;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// out[i][j] = in[pos[i]][pos[j]]: a matrix of a permuted numbering back in the natural one
template <typename T>
__global__ void dense_permute_kernel(int n, const int32_t* __restrict__ pos, const T* __restrict__ in, T* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * n) return;
  const int i = (int)(t / n), j = (int)(t - (int64_t)i * n);
  out[t] = in[(int64_t)pos[i] * n + pos[j]];
}

// ------------------------------------------------------------------------------------------ Cholesky
// Right-looking blocked Cholesky (lower, row-major, in place) with TB x TB tiles; tiles entirely outside
// the band stay zero and are skipped.
constexpr int TB = 32;
constexpr int CHOL_SMEM_MAX_N = 20000;  // x of a solve lives in shared memory (<= 160 KB in FP64)

// 1/d in FP64 from the FP32 reciprocal by two Newton-Raphson steps r <- r + r (1 - d r) (quadratic
// convergence: 2^-23 -> 2^-46 -> below FP64 rounding).  Used for the pivots of the factorisation, which
// lie well inside the FP32 range for stiffness matrices.
__device__ __forceinline__ double recip_newton(double d) {
  double r = (double)__frcp_rn((float)d);
  r = fma(r, fma(-d, r, 1.0), r);
  r = fma(r, fma(-d, r, 1.0), r);
  return r;
}

constexpr int CHOL_THREADS = 256;

// Diagonal tile kb, factored in shared memory by one CTA, right-looking in LDL^T form: at step k warp 0 forms
// the pivot reciprocal and the multipliers l_rk = T[r][k] / d_k of column k, then every thread updates
// T[r][c] -= l_rk T[c][k] over the live lower triangle (rows and columns > k), which is enumerated in packed
// order so that all warps but the last are full: one FP64 FMA per live element and no idle issue slots on a
// GPU whose FP64 rate (1/64 of FP32 on GB300) is the limit here.  The Cholesky factor L_unit sqrt(D) is
// written at the end, the square roots of all pivots taken together.  A non-positive pivot is recorded in
// *info and replaced by 1 so the sweep stays finite.
__device__ void chol_diag_tile(int n, double* A, int kb, int* info) {
  __shared__ double T[TB][TB + 1];
  __shared__ double ucol[TB];   // column k before scaling (d_k l_rk)
  __shared__ double dpiv[TB];
  const int k0 = kb * TB;
  const int nb = min(TB, n - k0);
  const int lane = threadIdx.x & 31;
  __syncthreads();              // the shared tile may still be read by a previous call of this CTA
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    T[r][c] = (r < nb && c < nb) ? A[(int64_t)(k0 + r) * n + k0 + c] : (r == c ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    // warp 0: pivot d_k and the multipliers l_rk = T[r][k] / d_k of column k (lane = row)
    if (threadIdx.x < 32) {
      double d = T[k][k];
      if (!(d > 0.0)) {
        if (lane == 0) atomicCAS(info, 0, k0 + k + 1);
        d = 1.0;
      }
      const double y = recip_newton(d);
      if (lane == 0) dpiv[k] = d;
      if (lane > k && lane < nb) {
        const double u = T[lane][k];
        ucol[lane] = u;
        T[lane][k] = u * y;
      }
    }
    __syncthreads();
    // trailing update of the lower triangle (rows and columns k+1 .. nb-1) in packed order, so that every
    // warp but the last is fully occupied: one FP64 FMA per element
    const int t = nb - 1 - k;
    const int m = t * (t + 1) / 2;
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
      int a = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
      if ((a + 1) * (a + 2) / 2 <= q) ++a;
      if (a * (a + 1) / 2 > q) --a;
      const int r = k + 1 + a, c = k + 1 + (q - a * (a + 1) / 2);
      T[r][c] = fma(-T[r][k], ucol[c], T[r][c]);
    }
    __syncthreads();
  }
  // Cholesky factor L = L_unit sqrt(D): column c scaled by sqrt(d_c) (all pivots at once)
  if (threadIdx.x < TB) dpiv[threadIdx.x] = threadIdx.x < nb ? sqrt(dpiv[threadIdx.x]) : 1.0;
  __syncthreads();
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    if (r < nb && c < nb) A[(int64_t)(k0 + r) * n + k0 + c] = c < r ? T[r][c] * dpiv[c] : (c == r ? dpiv[c] : 0.0);
  }
}

__global__ void __launch_bounds__(CHOL_THREADS) chol_diag_kernel(int n, double* A, int kb, int* info) {
  chol_diag_tile(n, A, kb, info);
}

// Panel: L[i, kb] = A[i, kb] L[kb,kb]^{-T} for the rows i below the diagonal tile within the band, one warp
// per row (lane c holds entry c; forward substitution with the reciprocal pivots, broadcast by shuffles).
constexpr int PANEL_WARPS = 8;
__device__ void chol_panel_block(int n, double* A, int kb, int bw, int blk) {
  __shared__ double L[TB][TB + 1];
  __shared__ double rp[TB];
  const int k0 = kb * TB;
  const int nb = min(TB, n - k0);
  __syncthreads();
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    L[r][c] = (r < nb && c < nb && c <= r) ? A[(int64_t)(k0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < TB) rp[threadIdx.x] = threadIdx.x < nb ? recip_newton(L[threadIdx.x][threadIdx.x]) : 0.0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int row = k0 + nb + blk * PANEL_WARPS + (threadIdx.x >> 5);
  if (row >= n || row - (k0 + nb - 1) > bw) return;   // whole warps exit together
  double x = lane < nb ? A[(int64_t)row * n + k0 + lane] : 0.0;
  for (int c = 0; c < nb; ++c) {
    if (lane == c) x *= rp[c];
    const double xc = __shfl_sync(0xffffffffu, x, c);
    if (lane > c) x = fma(-L[lane][c], xc, x);
  }
  if (lane < nb) A[(int64_t)row * n + k0 + lane] = x;
}

__global__ void __launch_bounds__(PANEL_WARPS * 32) chol_panel_kernel(int n, double* A, int kb, int bw) {
  chol_panel_block(n, A, kb, bw, blockIdx.x);
}

// Trailing update A[i][j] -= sum_q L[i][k0+q] L[j][k0+q] over the rows/columns below the diagonal tile within
// the band (j <= i), one 16 x 16 output tile per CTA (one element per thread).
constexpr int UT = 16;
__device__ void chol_update_tile(int n, double* A, int kb, int bw, int nt, int t) {
  __shared__ double Li[UT][TB + 1];
  __shared__ double Lj[UT][TB + 1];
  const int k0 = kb * TB;
  const int nb = min(TB, n - k0);
  const int base = k0 + nb;
  const int last = min(n - 1, k0 + nb - 1 + bw);   // last row with a nonzero in this block column
  __syncthreads();
  // lower-triangular tile enumeration: t -> (ti, tj), tj <= ti
  int ti = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
  while (ti * (ti + 1) / 2 > t) --ti;
  const int tj = t - ti * (ti + 1) / 2;
  if (ti >= nt) return;
  const int i0 = base + ti * UT, j0 = base + tj * UT;
  if (i0 > last || j0 > last) return;
  if (i0 - (j0 + UT - 1) > bw) return;            // tile entirely outside the band
  for (int e = threadIdx.x; e < UT * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    Li[r][c] = (i0 + r <= last && c < nb) ? A[(int64_t)(i0 + r) * n + k0 + c] : 0.0;
    Lj[r][c] = (j0 + r <= last && c < nb) ? A[(int64_t)(j0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  const int r = threadIdx.x / UT, c = threadIdx.x % UT;
  const int row = i0 + r, col = j0 + c;
  if (row > last || col > row || row - col > bw) return;
  double s = 0.0;
#pragma unroll 8
  for (int q = 0; q < TB; ++q) s = fma(Li[r][q], Lj[c][q], s);
  A[(int64_t)row * n + col] -= s;
}

__global__ void __launch_bounds__(UT * UT) chol_update_kernel(int n, double* A, int kb, int bw, int nt) {
  chol_update_tile(n, A, kb, bw, nt, blockIdx.x);
}

// The whole banded factorisation in one launch: one thread-block cluster of CHOL_CLUSTER CTAs steps through
// the tile columns (diagonal tile on CTA 0, panel rows and trailing-update tiles spread over the cluster),
// separated by the hardware cluster barrier (release/acquire, so the global writes of one phase are visible
// to the next).  One launch instead of three per tile column: on a busy GPU every launch waits for a free
// CTA slot, which made the 66 launches of the 675-dof factorisation take milliseconds behind a solve.
constexpr int CHOL_CLUSTER = 8;
static_assert(CHOL_THREADS == PANEL_WARPS * 32 && CHOL_THREADS == UT * UT, "one block size for all phases");

__device__ __forceinline__ void cluster_sync_all() {
  __threadfence();
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__global__ void __cluster_dims__(CHOL_CLUSTER, 1, 1) __launch_bounds__(CHOL_THREADS)
    chol_cluster_kernel(int n, double* A, int bw, int* info) {
  const int rank = blockIdx.x;   // the grid is one cluster
  const int nblk = (n + TB - 1) / TB;
  for (int kb = 0; kb < nblk; ++kb) {
    if (rank == 0) chol_diag_tile(n, A, kb, info);
    cluster_sync_all();
    const int k0 = kb * TB, nb = min(TB, n - k0);
    const int rows = min(n - (k0 + nb), bw);
    if (rows <= 0) continue;     // uniform: the last tile column
    const int pblocks = (rows + PANEL_WARPS - 1) / PANEL_WARPS;
    for (int pb = rank; pb < pblocks; pb += CHOL_CLUSTER) chol_panel_block(n, A, kb, bw, pb);
    cluster_sync_all();
    const int nt = (rows + UT - 1) / UT;
    for (int t = rank; t < nt * (nt + 1) / 2; t += CHOL_CLUSTER) chol_update_tile(n, A, kb, bw, nt, t);
    cluster_sync_all();
  }
}

// Inverses of the diagonal tiles of the factor, for the blocked triangular solves: Dinv[b] = L[b,b]^{-1}
// (lower triangular, row-major TB x TB, zero-padded for a ragged last tile).  One CTA per tile; warp w
// computes columns w, w+8, ... by forward substitution with lanes as rows.
template <typename T>
__global__ void __launch_bounds__(256) chol_block_inverse_kernel(int n, const double* __restrict__ L,
                                                                 T* __restrict__ Dinv) {
  __shared__ double Ls[TB][TB + 1];
  __shared__ double rp[TB];
  const int k0 = blockIdx.x * TB;
  const int nb = min(TB, n - k0);
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e / TB, c = e % TB;
    Ls[r][c] = (r < nb && c < nb && c <= r) ? L[(int64_t)(k0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < TB) rp[threadIdx.x] = threadIdx.x < nb ? recip_newton(Ls[threadIdx.x][threadIdx.x]) : 0.0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* D = Dinv + (int64_t)blockIdx.x * TB * TB;
  for (int j = warp; j < TB; j += 8) {
    double x = (lane == j) ? 1.0 : 0.0;
    for (int c = j; c < nb; ++c) {
      if (lane == c) x *= rp[c];
      const double xc = __shfl_sync(0xffffffffu, x, c);
      if (lane > c) x = fma(-Ls[lane][c], xc, x);
    }
    D[lane * TB + j] = (lane < nb && j < nb && lane >= j) ? (T)x : T(0);
  }
}

// FP32 inverse of a banded FP64 factor for the FP32 coarse solve: XT = (L^{-1})^T row by row, one warp
// per column c of L^{-1} (x = L^{-1} e_c by tiles: x_B = Dinv[b] (e_c - L[B, <B] x_<B), lanes as the rows of
// the tile), then Ainv = XT XT^T (= L^{-T} L^{-1}) by a tiled product.  L32 is the FP32 copy of the factor.
// The 8 warps of a CTA handle 8 consecutive columns, which share their first tile, so they walk the tiles
// together: each tile row of L (32 rows x the band) is staged once per CTA in shared memory (coalesced)
// and read from there by all 8 warps.
constexpr int TRINV_WARPS = 8;
constexpr int TRINV_PITCH_PAD = 1;   // odd row pitch: lanes (rows) hit distinct banks
__global__ void __launch_bounds__(TRINV_WARPS * 32) chol_trinv_f32_kernel(int n, const float* __restrict__ L32, int bw,
                                                                         const float* __restrict__ Dinv,
                                                                         float* __restrict__ XT) {
  extern __shared__ __align__(16) unsigned char c_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int c0 = blockIdx.x * nwarps;
  const int c = c0 + warp;
  const int span = bw + TB;                                  // band columns of a tile row, rounded up
  const int pitch = (span | 1) + TRINV_PITCH_PAD - 1;        // odd
  float* Ls = reinterpret_cast<float*>(c_smem);              // [TB][pitch]
  float* Dsm = Ls + TB * pitch;                              // [TB][TB + 1]: the tile inverse
  float* xall = Dsm + TB * (TB + 1);                         // [warps][n]
  float* x = xall + (size_t)warp * n;
  const int nblk = (n + TB - 1) / TB;
  const int bc = c0 / TB;                                    // first tile of every column of this CTA
  if (c < n) {
    float* out = XT + (int64_t)c * n;
    for (int i = lane; i < bc * TB; i += 32) out[i] = 0.f;
  }
  for (int kb = bc; kb < nblk; ++kb) {
    const int k0 = kb * TB;
    const int nb = min(TB, n - k0);
    const int jbeg = max(c0, k0 - bw);                       // leftmost column any warp of the CTA reads
    const int width = k0 - jbeg;                             // <= bw
    __syncthreads();                                          // previous tile row fully consumed
    for (int e = threadIdx.x; e < TB * width; e += blockDim.x) {
      const int r = e / width, j = e - r * width;
      Ls[r * pitch + j] = r < nb ? L32[(int64_t)(k0 + r) * n + jbeg + j] : 0.f;
    }
    for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) Dsm[(e / TB) * (TB + 1) + e % TB] = Dinv[(int64_t)kb * TB * TB + e];
    __syncthreads();
    if (c >= n) continue;
    const int i = k0 + lane;
    float t = 0.f;
    if (kb <= c / TB) {                                       // tiles up to the column's own: x = e_c there
      t = (i == c) ? 1.f : 0.f;
    } else if (lane < nb) {
      const float* Lr = Ls + lane * pitch - jbeg;
      float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;   // four independent chains
      int j = max(c, jbeg);
      for (; j + 4 <= k0; j += 4) {
        p0 = fmaf(Lr[j], x[j], p0);
        p1 = fmaf(Lr[j + 1], x[j + 1], p1);
        p2 = fmaf(Lr[j + 2], x[j + 2], p2);
        p3 = fmaf(Lr[j + 3], x[j + 3], p3);
      }
      for (; j < k0; ++j) p0 = fmaf(Lr[j], x[j], p0);
      t = -((p0 + p1) + (p2 + p3));
    }
    const float* D = Dsm + lane * (TB + 1);
    float acc = 0.f;
#pragma unroll 8
    for (int q = 0; q < TB; ++q) acc = fmaf(D[q], __shfl_sync(0xffffffffu, t, q), acc);
    if (lane < nb) {
      x[i] = acc;
      XT[(int64_t)c * n + i] = acc;
    }
    __syncwarp();
  }
}

// C = XT XT^T for an n x n row-major XT (upper triangular: XT[i][k] = 0 for k < i), 32 x 32 output tiles.
__global__ void __launch_bounds__(256) syrk_f32_kernel(int n, const float* __restrict__ XT, float* __restrict__ C) {
  __shared__ float As[32][33];
  __shared__ float Bs[32][33];
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 rows of 4 outputs each
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k0 = max(i0, j0) & ~31; k0 < n; k0 += 32) {
    for (int e = threadIdx.x; e < 32 * 32; e += 256) {
      const int r = e >> 5, q = e & 31;
      As[r][q] = (i0 + r < n && k0 + q < n) ? XT[(int64_t)(i0 + r) * n + k0 + q] : 0.f;
      Bs[r][q] = (j0 + r < n && k0 + q < n) ? XT[(int64_t)(j0 + r) * n + k0 + q] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < 32; ++q) {
      const float bv = Bs[tx][q];
#pragma unroll
      for (int m = 0; m < 4; ++m) acc[m] = fmaf(As[ty * 4 + m][q], bv, acc[m]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int i = i0 + ty * 4 + m, j = j0 + tx;
    if (i < n && j < n) C[(int64_t)i * n + j] = acc[m];
  }
}

// x = (L L^T)^{-1} b by one CTA with the tile inverses: forward, per tile b: t = x_B - L[B, <B] x_<B (warps
// over rows, lanes over the band columns), x_B = Dinv[b] t; backward, per tile (descending):
// x_B = Dinv[b]^T x_B, then x_j -= sum_{i in B} L[i][j] x_i for the band columns j before the tile.
template <typename T>
__global__ void __launch_bounds__(256) chol_solve_blocked_kernel(int n, const T* __restrict__ L, int bw,
                                                                 const T* __restrict__ Dinv,
                                                                 const T* __restrict__ b, T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char c_smem[];
  T* xs = reinterpret_cast<T*>(c_smem);
  __shared__ T Ds[TB][TB + 1];
  __shared__ T tv[TB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = b[i];
  const int nblk = (n + TB - 1) / TB;
  for (int kb = 0; kb < nblk; ++kb) {
    const int k0 = kb * TB;
    const int nb = min(TB, n - k0);
    const T* Dg = Dinv + (int64_t)kb * TB * TB;
    for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) Ds[e / TB][e % TB] = Dg[e];
    __syncthreads();
    const int jbeg = max(0, k0 - bw);
    for (int rr = warp; rr < nb; rr += 8) {
      const T* Lr = L + (int64_t)(k0 + rr) * n;
      T acc = T(0);
      for (int j = jbeg + lane; j < k0; j += 32) acc += Lr[j] * xs[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) tv[rr] = xs[k0 + rr] - acc;
    }
    __syncthreads();
    if (warp == 0 && lane < nb) {
      T acc = T(0);
      for (int c = 0; c <= lane; ++c) acc += Ds[lane][c] * tv[c];
      xs[k0 + lane] = acc;
    }
    __syncthreads();
  }
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * TB;
    const int nb = min(TB, n - k0);
    const T* Dg = Dinv + (int64_t)kb * TB * TB;
    for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) Ds[e / TB][e % TB] = Dg[e];
    if (threadIdx.x < TB) tv[threadIdx.x] = threadIdx.x < nb ? xs[k0 + threadIdx.x] : T(0);
    __syncthreads();
    if (warp == 0 && lane < nb) {
      T acc = T(0);
      for (int r = lane; r < nb; ++r) acc += Ds[r][lane] * tv[r];
      xs[k0 + lane] = acc;
    }
    __syncthreads();
    const int jbeg = max(0, k0 - bw);
    for (int j = jbeg + threadIdx.x; j < k0; j += blockDim.x) {
      T acc = T(0);
      for (int r = 0; r < nb; ++r) acc += L[(int64_t)(k0 + r) * n + j] * xs[k0 + r];
      xs[j] -= acc;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xs[i];
}

// x = (L L^T)^{-1} x in place (x in shared memory) for a banded lower factor, by one CTA: forward then
// backward substitution in TB blocks; a warp solves each diagonal block, the CTA updates the band rows.
// `first` skips the leading blocks of x known to be zero (the right-hand side e_j of the inverse).
template <typename T>
__device__ void chol_solve_smem(int n, const T* __restrict__ L, int bw, T* x, int first) {
  const int kstart = (first / TB) * TB;
  for (int k0 = kstart; k0 < n; k0 += TB) {
    const int nb = min(TB, n - k0);
    if (threadIdx.x < 32) {
      // lane r holds row r of the diagonal block in registers; the block is solved by shuffles
      const int lane = threadIdx.x;
      T xr = lane < nb ? x[k0 + lane] : T(0);
      T Lrow[TB];
#pragma unroll
      for (int c = 0; c < TB; ++c)
        Lrow[c] = (lane < nb && c <= lane) ? L[(int64_t)(k0 + lane) * n + k0 + c] : T(0);
      const T rinv = lane < nb ? T(1) / L[(int64_t)(k0 + lane) * n + k0 + lane] : T(0);
#pragma unroll
      for (int k = 0; k < TB; ++k) {
        if (k < nb) {
          const T xk = __shfl_sync(0xffffffffu, xr, k) * __shfl_sync(0xffffffffu, rinv, k);
          if (lane == k) xr = xk;
          if (lane > k) xr -= Lrow[k] * xk;
        }
      }
      if (lane < nb) x[k0 + lane] = xr;
    }
    __syncthreads();
    const int rend = min(n, k0 + nb + bw);
    for (int r = k0 + nb + threadIdx.x; r < rend; r += blockDim.x) {
      T acc = T(0);
      const T* Lr = L + (int64_t)r * n + k0;
      for (int c = 0; c < nb; ++c) acc += Lr[c] * x[k0 + c];
      x[r] -= acc;
    }
    __syncthreads();
  }
  const int nblk = (n + TB - 1) / TB;
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * TB;
    const int nb = min(TB, n - k0);
    if (threadIdx.x < 32) {
      // lane c holds column c of the diagonal block (L^T is solved by columns)
      const int lane = threadIdx.x;
      T xr = lane < nb ? x[k0 + lane] : T(0);
      T Lcol[TB];
#pragma unroll
      for (int r = 0; r < TB; ++r)
        Lcol[r] = (lane < nb && r < nb && r >= lane) ? L[(int64_t)(k0 + r) * n + k0 + lane] : T(0);
      const T rinv = lane < nb ? T(1) / L[(int64_t)(k0 + lane) * n + k0 + lane] : T(0);
#pragma unroll
      for (int k = TB - 1; k >= 0; --k) {
        if (k < nb) {
          const T xk = __shfl_sync(0xffffffffu, xr, k) * __shfl_sync(0xffffffffu, rinv, k);
          if (lane == k) xr = xk;
          if (lane < k) xr -= Lcol[k] * xk;
        }
      }
      if (lane < nb) x[k0 + lane] = xr;
    }
    __syncthreads();
    const int cbeg = max(0, k0 - bw);
    for (int c = cbeg + threadIdx.x; c < k0; c += blockDim.x) {
      T acc = T(0);
      for (int r = 0; r < nb; ++r) acc += L[(int64_t)(k0 + r) * n + c] * x[k0 + r];
      x[c] -= acc;
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(256) chol_solve_kernel(int n, const T* __restrict__ L, int bw, const T* __restrict__ b,
                                                        T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char c_smem[];
  T* xs = reinterpret_cast<T*>(c_smem);
  for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = b[i];
  __syncthreads();
  chol_solve_smem<T>(n, L, bw, xs, 0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xs[i];
}

// Row j of A^{-1} (= column j, A symmetric) by one CTA per row: solve A x = e_j with the factor.
__global__ void __launch_bounds__(256) chol_inverse_kernel(int n, const double* __restrict__ L, int bw,
                                                          double* __restrict__ Ainv) {
  extern __shared__ __align__(16) unsigned char c_smem[];
  double* xs = reinterpret_cast<double*>(c_smem);
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = i == j ? 1.0 : 0.0;
  __syncthreads();
  chol_solve_smem<double>(n, L, bw, xs, j);
  double* row = Ainv + (int64_t)j * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) row[i] = xs[i];
}

// y = A x for a dense row-major n x n matrix, one warp per row (coalesced along the row).
template <typename T>
__global__ void dense_gemv_kernel(int n, const T* __restrict__ A, const T* __restrict__ x, T* __restrict__ y) {
  const int warp = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const T* row = A + (int64_t)warp * n;
  double acc = 0.0;
  for (int c = lane; c < n; c += 32) acc = fma((double)row[c], (double)x[c], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[warp] = (T)acc;
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
  if (nnodes < 0 || dim < 1 || dim > 3 || !bcmask || !x || !y) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (nnodes == 0) return PMG_OK;
  const unsigned g = blocks_for(nnodes, 256);
  if (dtype == PMG_F64 && dim == 1)
    mask_bc_kernel<double, 1><<<g, 256, 0, st>>>(nnodes, bcmask, keep_bc, (const double*)x, (double*)y);
  else if (dtype == PMG_F32 && dim == 1)
    mask_bc_kernel<float, 1><<<g, 256, 0, st>>>(nnodes, bcmask, keep_bc, (const float*)x, (float*)y);
  else if (dtype == PMG_F64 && dim == 3)
    mask_bc_kernel<double, 3><<<g, 256, 0, st>>>(nnodes, bcmask, keep_bc, (const double*)x, (double*)y);
  else if (dtype == PMG_F64)
    mask_bc_kernel<double, 2><<<g, 256, 0, st>>>(nnodes, bcmask, keep_bc, (const double*)x, (double*)y);
  else if (dtype == PMG_F32 && dim == 3)
    mask_bc_kernel<float, 3><<<g, 256, 0, st>>>(nnodes, bcmask, keep_bc, (const float*)x, (float*)y);
  else if (dtype == PMG_F32)
    mask_bc_kernel<float, 2><<<g, 256, 0, st>>>(nnodes, bcmask, keep_bc, (const float*)x, (float*)y);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_split_bc(int dtype, int dim, int64_t nnodes, const uint8_t* bcmask, double bcdiag, const void* rhs,
                 void* direct, void* free_part, const void* cdiag, void* stream) {
  if (nnodes < 0 || dim < 1 || dim > 3 || !bcmask || !rhs || !direct || !free_part || !(bcdiag != 0.0))
    return PMG_BAD_ARG;
  if (nnodes == 0) return PMG_OK;
  cudaStream_t st = as_stream(stream);
  const unsigned g = blocks_for(nnodes, 256);
  if (dtype == PMG_F64 && dim == 1) {
    split_bc_kernel<double, 1><<<g, 256, 0, st>>>(nnodes, bcmask, bcdiag, (const double*)rhs, (double*)direct,
                                                 (double*)free_part, (const double*)cdiag);
    return check_launch();
  }
  if (dtype == PMG_F32 && dim == 1) {
    split_bc_kernel<float, 1><<<g, 256, 0, st>>>(nnodes, bcmask, (float)(bcdiag), (const float*)rhs,
                                                (float*)direct, (float*)free_part, (const float*)cdiag);
    return check_launch();
  }
  if (dtype == PMG_F64 && dim == 3)
    split_bc_kernel<double, 3><<<g, 256, 0, st>>>(nnodes, bcmask, bcdiag, (const double*)rhs, (double*)direct,
                                                 (double*)free_part, (const double*)cdiag);
  else if (dtype == PMG_F64)
    split_bc_kernel<double, 2><<<g, 256, 0, st>>>(nnodes, bcmask, bcdiag, (const double*)rhs, (double*)direct,
                                                 (double*)free_part, (const double*)cdiag);
  else if (dtype == PMG_F32 && dim == 3)
    split_bc_kernel<float, 3><<<g, 256, 0, st>>>(nnodes, bcmask, (float)(bcdiag), (const float*)rhs,
                                                (float*)direct, (float*)free_part, (const float*)cdiag);
  else if (dtype == PMG_F32)
    split_bc_kernel<float, 2><<<g, 256, 0, st>>>(nnodes, bcmask, (float)(bcdiag), (const float*)rhs,
                                                (float*)direct, (float*)free_part, (const float*)cdiag);
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

int pmg_convert_dscale(int src_dtype, int dst_dtype, int64_t n, const void* x, void* y, const double* s, int inverse,
                       void* stream) {
  if (n < 0 || !x || !y || !s) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const unsigned g = stream_blocks(n);
  if (src_dtype == PMG_F64 && dst_dtype == PMG_F32)
    convert_dscale_kernel<double, float><<<g, 256, 0, st>>>(n, (const double*)x, (float*)y, s, inverse);
  else if (src_dtype == PMG_F32 && dst_dtype == PMG_F64)
    convert_dscale_kernel<float, double><<<g, 256, 0, st>>>(n, (const float*)x, (double*)y, s, inverse);
  else if (src_dtype == PMG_F64 && dst_dtype == PMG_F64)
    convert_dscale_kernel<double, double><<<g, 256, 0, st>>>(n, (const double*)x, (double*)y, s, inverse);
  else if (src_dtype == PMG_F32 && dst_dtype == PMG_F32)
    convert_dscale_kernel<float, float><<<g, 256, 0, st>>>(n, (const float*)x, (float*)y, s, inverse);
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

int pmg_cheb_coeffs(const double* lmax_dev, double lmax_host, double ratio, int degree, double* coef, void* stream) {
  if (degree < 1 || degree > 64 || !(ratio > 1.0) || !coef) return PMG_BAD_ARG;
  cheb_coeffs_kernel<<<1, 32, 0, as_stream(stream)>>>(lmax_dev, lmax_host, ratio, degree, coef);
  return check_launch();
}

int pmg_cheb_step(int dtype, int64_t n, const void* r, const void* diag, void* d, void* x, const double* coef, int step,
                  int init, void* stream) {
  if (n < 0 || !r || !diag || !d || !x || !coef || step < 0 || step >= 64) return PMG_BAD_ARG;
  if (n == 0) return PMG_OK;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    cheb_step_kernel<double><<<stream_blocks(n), 256, 0, st>>>(n, (const double*)r, (const double*)diag, (double*)d,
                                                              (double*)x, coef, step, init);
  else if (dtype == PMG_F32)
    cheb_step_kernel<float><<<stream_blocks(n), 256, 0, st>>>(n, (const float*)r, (const float*)diag, (float*)d,
                                                             (float*)x, coef, step, init);
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
  static int cluster_ok[64] = {0};   // 0 unknown, 1 yes, -1 no
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    if (cluster_ok[dev] == 0) {
      int v = 0;
      cudaDeviceGetAttribute(&v, cudaDevAttrClusterLaunch, dev);
      cluster_ok[dev] = v ? 1 : -1;
    }
    if (cluster_ok[dev] > 0) {
      chol_cluster_kernel<<<CHOL_CLUSTER, CHOL_THREADS, 0, st>>>(n, A, bw, info);
      return check_launch();
    }
  }
  const int nblk = (n + TB - 1) / TB;
  for (int kb = 0; kb < nblk; ++kb) {
    chol_diag_kernel<<<1, CHOL_THREADS, 0, st>>>(n, A, kb, info);
    const int k0 = kb * TB, nb = min(TB, n - k0);
    const int rows = min(n - (k0 + nb), bw);      // band rows below the tile
    if (rows <= 0) continue;
    chol_panel_kernel<<<(rows + PANEL_WARPS - 1) / PANEL_WARPS, PANEL_WARPS * 32, 0, st>>>(n, A, kb, bw);
    const int nt = (rows + UT - 1) / UT;
    chol_update_kernel<<<nt * (nt + 1) / 2, UT * UT, 0, st>>>(n, A, kb, bw, nt);
    const int rc = check_launch();
    if (rc != PMG_OK) return rc;
  }
  return check_launch();
}

int pmg_cholesky_block_inverses(int dtype, int n, const double* L, void* Dinv, void* stream) {
  if (n <= 0 || !L || !Dinv || (const void*)L == Dinv) return PMG_BAD_ARG;
  const int nblk = (n + TB - 1) / TB;
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    chol_block_inverse_kernel<double><<<nblk, 256, 0, st>>>(n, L, (double*)Dinv);
  else if (dtype == PMG_F32)
    chol_block_inverse_kernel<float><<<nblk, 256, 0, st>>>(n, L, (float*)Dinv);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_dense_permute(int dtype, int n, const int32_t* pos, const void* in, void* out, void* stream) {
  if (n <= 0 || !pos || !in || !out || in == out) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const int64_t nn = (int64_t)n * n;
  if (dtype == PMG_F64)
    dense_permute_kernel<double><<<blocks_for(nn, 256), 256, 0, st>>>(n, pos, (const double*)in, (double*)out);
  else if (dtype == PMG_F32)
    dense_permute_kernel<float><<<blocks_for(nn, 256), 256, 0, st>>>(n, pos, (const float*)in, (float*)out);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

size_t pmg_cholesky_inverse_f32_scratch_bytes(int n) {
  if (n <= 0) return 0;
  const size_t nblk = (size_t)(n + TB - 1) / TB;
  return sizeof(float) * ((size_t)n * n * 2 + nblk * TB * TB);
}

int pmg_cholesky_inverse_f32(int n, const double* L, int bw, void* scratch, float* Ainv, void* stream) {
  if (n <= 0 || n > CHOL_SMEM_MAX_N || !L || !scratch || !Ainv || bw < 0) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const int nblk = (n + TB - 1) / TB;
  float* L32 = reinterpret_cast<float*>(scratch);
  float* XT = L32 + (size_t)n * n;
  float* Dinv = XT + (size_t)n * n;
  chol_block_inverse_kernel<float><<<nblk, 256, 0, st>>>(n, L, Dinv);
  convert_kernel<double, float><<<stream_blocks((int64_t)n * n), 256, 0, st>>>((int64_t)n * n, L, L32, 1.0);
  // shared memory: one staged tile row of L (TB x odd pitch >= bw + TB) and one column per warp (up to 8
  // warps, fewer when the columns do not fit)
  const int pitch = ((bw + TB) | 1) + TRINV_PITCH_PAD - 1;
  const size_t tile_bytes = sizeof(float) * ((size_t)TB * pitch + TB * (TB + 1)), col_bytes = sizeof(float) * (size_t)n;
  const size_t budget = 200 * 1024;
  if (tile_bytes + col_bytes > budget) return PMG_BAD_ARG;
  const int warps = (int)std::min<size_t>(TRINV_WARPS, (budget - tile_bytes) / col_bytes);
  const size_t smem = tile_bytes + col_bytes * warps;
  static size_t smem_set[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch();
  if (smem > smem_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(chol_trinv_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      return PMG_CUDA_ERR;
    }
    smem_set[dev] = smem;
  }
  chol_trinv_f32_kernel<<<(n + warps - 1) / warps, warps * 32, smem, st>>>(n, L32, bw, Dinv, XT);
  const dim3 grid(nblk, nblk);
  syrk_f32_kernel<<<grid, 256, 0, st>>>(n, XT, Ainv);
  return check_launch();
}

int pmg_cholesky_solve_blocked(int dtype, int n, const void* L, int bw, const void* Dinv, const void* b, void* x,
                               void* stream) {
  if (n <= 0 || n > CHOL_SMEM_MAX_N || !L || !Dinv || !b || !x || bw < 0 || b == x) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const size_t smem = (dtype == PMG_F64 ? sizeof(double) : sizeof(float)) * (size_t)n;
  cudaError_t e = cudaSuccess;
  // the opt-in above the default dynamic shared memory limit, raised once per size (x lives in smem)
  static size_t smem_set[2][64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch();
  const int ti = dtype == PMG_F64 ? 0 : 1;
  if (dtype == PMG_F64) {
    if (smem > smem_set[ti][dev]) {
      e = cudaFuncSetAttribute(chol_solve_blocked_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess) smem_set[ti][dev] = smem;
    }
    if (e == cudaSuccess)
      chol_solve_blocked_kernel<double><<<1, 256, smem, st>>>(n, (const double*)L, bw, (const double*)Dinv,
                                                              (const double*)b, (double*)x);
  } else if (dtype == PMG_F32) {
    if (smem > smem_set[ti][dev]) {
      e = cudaFuncSetAttribute(chol_solve_blocked_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess) smem_set[ti][dev] = smem;
    }
    if (e == cudaSuccess)
      chol_solve_blocked_kernel<float><<<1, 256, smem, st>>>(n, (const float*)L, bw, (const float*)Dinv,
                                                             (const float*)b, (float*)x);
  } else {
    return PMG_BAD_ARG;
  }
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return check_launch();
}

int pmg_cholesky_inverse(int n, const double* L, int bw, double* Ainv, void* stream) {
  if (n <= 0 || n > CHOL_SMEM_MAX_N || !L || !Ainv || bw < 0 || (const void*)L == (const void*)Ainv) return PMG_BAD_ARG;
  const size_t smem = sizeof(double) * (size_t)n;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(chol_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      return PMG_CUDA_ERR;
    }
  }
  chol_inverse_kernel<<<(unsigned)n, 256, smem, as_stream(stream)>>>(n, L, bw, Ainv);
  return check_launch();
}

int pmg_dense_gemv(int dtype, int n, const void* A, const void* x, void* y, void* stream) {
  if (n <= 0 || !A || !x || !y || x == y) return PMG_BAD_ARG;
  const unsigned blocks = (unsigned)(((int64_t)n * 32 + 255) / 256);
  cudaStream_t st = as_stream(stream);
  if (dtype == PMG_F64)
    dense_gemv_kernel<double><<<blocks, 256, 0, st>>>(n, (const double*)A, (const double*)x, (double*)y);
  else if (dtype == PMG_F32)
    dense_gemv_kernel<float><<<blocks, 256, 0, st>>>(n, (const float*)A, (const float*)x, (float*)y);
  else
    return PMG_BAD_ARG;
  return check_launch();
}

int pmg_cholesky_solve(int dtype, int n, const void* L, int bw, const void* b, void* x, void* stream) {
  if (n <= 0 || n > CHOL_SMEM_MAX_N || !L || !b || !x || bw < 0 || b == x) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  const size_t smem = (dtype == PMG_F64 ? sizeof(double) : sizeof(float)) * (size_t)n;
  cudaError_t e = cudaSuccess;
  if (dtype == PMG_F64) {
    if (smem > 48 * 1024)
      e = cudaFuncSetAttribute(chol_solve_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      chol_solve_kernel<double><<<1, 256, smem, st>>>(n, (const double*)L, bw, (const double*)b, (double*)x);
  } else if (dtype == PMG_F32) {
    if (smem > 48 * 1024)
      e = cudaFuncSetAttribute(chol_solve_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      chol_solve_kernel<float><<<1, 256, smem, st>>>(n, (const float*)L, bw, (const float*)b, (float*)x);
  } else {
    return PMG_BAD_ARG;
  }
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return check_launch();
}

}  // extern "C"
