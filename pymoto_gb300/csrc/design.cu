// Design-variable kernels: density filters and their adjoints, SIMP, the adjoint sensitivity contraction
// and the optimality-criteria update.  All FP64 (these streams are small next to the solve).
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace pmg {

// ------------------------------------------------------------------------------------------ DensityFilter
// Cone weights max(0, r - |d|) over the window int(r) (element-index distances).
__device__ __forceinline__ double cone(double r, int dx, int dy, int dz) {
  const double d = sqrt((double)(dx * dx + dy * dy + dz * dz));
  return r - d > 0.0 ? r - d : 0.0;
}

__device__ __forceinline__ void elem_ijk(const Grid& g, int64_t e64, int& i, int& j, int& k) {
  const unsigned e = (unsigned)e64, nx = (unsigned)g.nx, ny = (unsigned)g.ny;
  const unsigned t = e / nx;
  i = (int)(e - t * nx);
  k = (int)(t / ny);
  j = (int)(t - (unsigned)k * ny);
}

__global__ void density_rowsum_kernel(Grid g, double r, double* __restrict__ s) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  int i, j, k;
  elem_ijk(g, e, i, j, k);
  const int d = (int)r;
  const int dzr = g.nz == 0 ? 0 : d;
  double acc = 0.0;
  for (int dz = -dzr; dz <= dzr; ++dz) {
    const int kk = k + dz;
    if (kk < 0 || kk >= g.ez()) continue;
    for (int dy = -d; dy <= d; ++dy) {
      const int jj = j + dy;
      if (jj < 0 || jj >= g.ny) continue;
      for (int dx = -d; dx <= d; ++dx) {
        const int ii = i + dx;
        if (ii < 0 || ii >= g.nx) continue;
        acc += cone(r, dx, dy, dz);
      }
    }
  }
  s[e] = acc;
}

// forward: y_i = sum_j H_ij x_j / s_i ;  transpose: y_j = sum_i H_ij (x_i / s_i)  (H symmetric)
template <bool TRANSPOSE>
__global__ void density_filter_kernel(Grid g, double r, const double* __restrict__ s, const double* __restrict__ x,
                                      double* __restrict__ y) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  int i, j, k;
  elem_ijk(g, e, i, j, k);
  const int d = (int)r;
  const int dzr = g.nz == 0 ? 0 : d;
  double acc = 0.0;
  for (int dz = -dzr; dz <= dzr; ++dz) {
    const int kk = k + dz;
    if (kk < 0 || kk >= g.ez()) continue;
    for (int dy = -d; dy <= d; ++dy) {
      const int jj = j + dy;
      if (jj < 0 || jj >= g.ny) continue;
      for (int dx = -d; dx <= d; ++dx) {
        const int ii = i + dx;
        if (ii < 0 || ii >= g.nx) continue;
        const int64_t m = elem_id(g, ii, jj, kk);
        const double v = TRANSPOSE ? x[m] / s[m] : x[m];
        acc = fma(cone(r, dx, dy, dz), v, acc);
      }
    }
  }
  y[e] = TRANSPOSE ? acc : acc / s[e];
}

// ------------------------------------------------------------------------------------------ FilterConv
// Forward: y[o] = sum_m w[m] x[pad(o + (K-1) - m)]  (kernel flipped: 'valid' convolution); pad maps may hold -1
// for the positions of constant-value sides, which contribute nothing here.
__global__ void conv_filter_kernel(Grid g, const double* __restrict__ w, int kx, int ky, int kz,
                                   const int32_t* __restrict__ px, const int32_t* __restrict__ py,
                                   const int32_t* __restrict__ pz, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  int i, j, k;
  elem_ijk(g, e, i, j, k);
  double acc = 0.0;
  for (int c = 0; c < kz; ++c) {
    const int kk = pz[k + (kz - 1) - c];
    if (kk < 0) continue;   // padded position of a constant-value side: its value enters as a separate field
    for (int b = 0; b < ky; ++b) {
      const int jj = py[j + (ky - 1) - b];
      if (jj < 0) continue;
      const double* wr = w + ((int64_t)0 * ky + b) * kz + c;
      for (int a = 0; a < kx; ++a) {
        const int ii = px[i + (kx - 1) - a];
        if (ii < 0) continue;
        acc = fma(wr[(int64_t)a * ky * kz], x[elem_id(g, ii, jj, kk)], acc);
      }
    }
  }
  y[e] = acc;
}

// Adjoint, gather form: dx[j] = sum over padded positions P with pad(P) = j of sum_m w[m] d[P - (K-1) + m]
// (the output o = P - (K-1) + m must lie inside the grid).  The padded positions of index j along each
// axis are inv_pos[inv_ptr[j] .. inv_ptr[j+1]) (inverse of the pad map, built on the host).
__global__ void conv_filter_adjoint_kernel(Grid g, const double* __restrict__ w, int kx, int ky, int kz,
                                           const int32_t* __restrict__ xp, const int32_t* __restrict__ xs,
                                           const int32_t* __restrict__ yp, const int32_t* __restrict__ ys,
                                           const int32_t* __restrict__ zp, const int32_t* __restrict__ zs,
                                           const double* __restrict__ d, double* __restrict__ y) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  int i, j, k;
  elem_ijk(g, e, i, j, k);
  const int ez = g.ez();
  double acc = 0.0;
  for (int qz = zp[k]; qz < zp[k + 1]; ++qz) {
    const int Pz = zs[qz];
    for (int qy = yp[j]; qy < yp[j + 1]; ++qy) {
      const int Py = ys[qy];
      for (int qx = xp[i]; qx < xp[i + 1]; ++qx) {
        const int Px = xs[qx];
        for (int c = 0; c < kz; ++c) {
          const int oz = Pz - (kz - 1) + c;
          if (oz < 0 || oz >= ez) continue;
          for (int b = 0; b < ky; ++b) {
            const int oy = Py - (ky - 1) + b;
            if (oy < 0 || oy >= g.ny) continue;
            for (int a = 0; a < kx; ++a) {
              const int ox = Px - (kx - 1) + a;
              if (ox < 0 || ox >= g.nx) continue;
              acc = fma(w[((int64_t)a * ky + b) * kz + c], d[elem_id(g, ox, oy, oz)], acc);
            }
          }
        }
      }
    }
  }
  y[e] = acc;
}

// ------------------------------------------------------------------------------------------ SIMP
__global__ void simp_kernel(int64_t n, double xmin, double p, const double* __restrict__ x, double* __restrict__ y,
                            float* __restrict__ y32) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xi = x[i];
  const double xp = p == 3.0 ? xi * xi * xi : pow(xi, p);
  const double v = xmin + (1.0 - xmin) * xp;
  if (y) y[i] = v;
  if (y32) y32[i] = (float)v;
}

__global__ void simp_backward_kernel(int64_t n, double xmin, double p, const double* __restrict__ x,
                                     const double* __restrict__ dy, double* __restrict__ dx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xi = x[i];
  const double xp = p == 3.0 ? xi * xi : pow(xi, p - 1.0);
  dx[i] = dy[i] * (p * (1.0 - xmin) * xp);
}

// ------------------------------------------------------------------------------------------ sensitivity
// dx_e (+)= alpha * u_e^T K0 v_e with Dirichlet entries zeroed; one thread per element.
template <int DIM>
__global__ void sens_kernel(Grid g, ElemMat<double, Traits<DIM>::NDE> K0, const uint8_t* __restrict__ bcmask,
                            const double* __restrict__ u, const double* __restrict__ v, double alpha, int accumulate,
                            double* __restrict__ dx) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  int i, j, k;
  elem_ijk(g, e, i, j, k);
  double ue[NDE], ve[NDE];
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    const int64_t nd = node_id(g, i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1));
    const uint8_t m = bcmask ? bcmask[nd] : 0;
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const bool bc = (m >> c) & 1;
      ue[a * DIM + c] = bc ? 0.0 : u[nd * DIM + c];
      ve[a * DIM + c] = bc ? 0.0 : v[nd * DIM + c];
    }
  }
  double s = 0.0;
#pragma unroll
  for (int r = 0; r < NDE; ++r) {
    double t = 0.0;
#pragma unroll
    for (int c = 0; c < NDE; ++c) t = fma(K0.v[r * NDE + c], ve[c], t);
    s = fma(ue[r], t, s);
  }
  const double val = alpha * s;
  dx[e] = accumulate ? dx[e] + val : val;
}

// Mixed-precision contraction for the mixed solver path: the element vectors are shifted (in FP64) by the
// value at their first node per component (K0 annihilates rigid translations, so the shift is exact), the
// differences are rounded to FP32 and the 24 x 24 quadratic form runs in FP32 (FP32 K0 as a uniform
// operand); only the result returns to FP64.  The error is that of FP32 arithmetic on the deformation of the
// element, not on its displacement.
template <int DIM>
__global__ void sens_mixed_kernel(Grid g, ElemMat<float, Traits<DIM>::NDE> K0, const uint8_t* __restrict__ bcmask,
                                  const double* __restrict__ u, const double* __restrict__ v, double alpha,
                                  int accumulate, double* __restrict__ dx) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  int i, j, k;
  elem_ijk(g, e, i, j, k);
  double ud[NDE], vd[NDE];
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    const int64_t nd = node_id(g, i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1));
    const uint8_t m = bcmask ? bcmask[nd] : 0;
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const bool bc = (m >> c) & 1;
      ud[a * DIM + c] = bc ? 0.0 : u[nd * DIM + c];
      vd[a * DIM + c] = bc ? 0.0 : v[nd * DIM + c];
    }
  }
  float uf[NDE], vf[NDE];
#pragma unroll
  for (int q = 0; q < NDE; ++q) {
    uf[q] = (float)(ud[q] - ud[q % DIM]);
    vf[q] = (float)(vd[q] - vd[q % DIM]);
  }
  float s = 0.f;
#pragma unroll
  for (int r = 0; r < NDE; ++r) {
    float t = 0.f;
#pragma unroll
    for (int c = 0; c < NDE; ++c) t = fmaf(K0.v[r * NDE + c], vf[c], t);
    s = fmaf(uf[r], t, s);
  }
  const double val = alpha * (double)s;
  dx[e] = accumulate ? dx[e] + val : val;
}

// Tiled form of the mixed-precision contraction (3D): a CTA owns 32 x 8 elements per layer and walks a chunk
// of z layers.  Each staged node is shifted once by a reference displacement of the tile in FP64 and split
// into an FP32 pair hi + lo (5 FP64 operations per value and node, instead of 2 per value and element); the
// element differences (hi_a - hi_0) + (lo_a - lo_0) are then formed in FP32 with the accuracy of the FP64
// shift, and the quadratic form runs in FP32 as above.
constexpr int SENS_TX = 32, SENS_TY = 8, SENS_NX = SENS_TX + 1, SENS_NY = SENS_TY + 1;
constexpr int SENS_PLANE = SENS_NX * SENS_NY;

__global__ void __launch_bounds__(SENS_TX * SENS_TY)
    sens_mixed_tiled_kernel(Grid g, ElemMat<float, 24> K0, const uint8_t* __restrict__ bcmask,
                            const double* __restrict__ u, const double* __restrict__ v, double alpha, int accumulate,
                            int zchunk, double* __restrict__ dx) {
  __shared__ float sh[2][4][3][SENS_PLANE];     // [layer parity][u_hi, u_lo, v_hi, v_lo][component][node]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int i0 = blockIdx.x * SENS_TX, j0 = blockIdx.y * SENS_TY;
  const int kb = blockIdx.z * zchunk, ke = min(g.nz, kb + zchunk);
  if (kb >= ke) return;
  const int nnx = g.nx + 1, nny = g.ny + 1;
  double cu[3], cv[3];
  {
    const int64_t n0 = node_id(g, i0, j0, kb);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      cu[d] = u[n0 * 3 + d];
      cv[d] = v[n0 * 3 + d];
    }
  }
  auto stage = [&](int k, int buf) {
    for (int q = tid; q < SENS_PLANE; q += SENS_TX * SENS_TY) {
      const int cy = q / SENS_NX, cx = q - cy * SENS_NX;
      const int gi = i0 + cx, gj = j0 + cy;
      if (gi < nnx && gj < nny) {
        const int64_t nd = node_id(g, gi, gj, k);
        const unsigned m = bcmask ? bcmask[nd] : 0u;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const bool bc = (m >> d) & 1u;
          const double du = (bc ? 0.0 : u[nd * 3 + d]) - cu[d];
          const double dv = (bc ? 0.0 : v[nd * 3 + d]) - cv[d];
          const float hu = (float)du, hv = (float)dv;
          sh[buf][0][d][q] = hu;
          sh[buf][1][d][q] = (float)(du - (double)hu);
          sh[buf][2][d][q] = hv;
          sh[buf][3][d][q] = (float)(dv - (double)hv);
        }
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) sh[buf][0][d][q] = sh[buf][1][d][q] = sh[buf][2][d][q] = sh[buf][3][d][q] = 0.f;
      }
    }
  };
  const int ei = i0 + lane, ej = j0 + warp;
  const bool inside = ei < g.nx && ej < g.ny;
  stage(kb, kb & 1);
  for (int k = kb; k < ke; ++k) {
    stage(k + 1, (k + 1) & 1);
    __syncthreads();
    if (inside) {
      float uf[24], vf[24];
      const int p00 = warp * SENS_NX + lane;
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int buf = (k + ((a >> 2) & 1)) & 1;
        const int p = p00 + ((a >> 1) & 1) * SENS_NX + (a & 1);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          uf[a * 3 + d] = (sh[buf][0][d][p] - sh[k & 1][0][d][p00]) + (sh[buf][1][d][p] - sh[k & 1][1][d][p00]);
          vf[a * 3 + d] = (sh[buf][2][d][p] - sh[k & 1][2][d][p00]) + (sh[buf][3][d][p] - sh[k & 1][3][d][p00]);
        }
      }
      float s = 0.f;
#pragma unroll
      for (int r = 0; r < 24; ++r) {
        float t = 0.f;
#pragma unroll
        for (int c = 0; c < 24; ++c) t = fmaf(K0.v[r * 24 + c], vf[c], t);
        s = fmaf(uf[r], t, s);
      }
      const int64_t e = elem_id(g, ei, ej, k);
      const double val = alpha * (double)s;
      dx[e] = accumulate ? dx[e] + val : val;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------ OC update
// State in scratch: sum partials and the bisection interval, all on the device.
// x sqrt(-dg/lmid) is evaluated as (x sqrt(-dg)) / sqrt(lmid): the per-element square root is taken once and
// each bisection step costs one multiply and a clip per element (the two forms differ in the last bits).
constexpr int OC_THREADS = 256;
constexpr int OC_MAX_BLOCKS = 1024;
constexpr int OC_TREE = 5;                      // bisection levels resolved per pass of the single launch
constexpr int OC_CAND = (1 << OC_TREE) - 1;     // midpoints of a depth-5 bisection tree
struct OCScratch {
  double partial[OC_MAX_BLOCKS];
  double l1, l2, lmid, lmid_last;
  unsigned int ticket;
  unsigned int generation, error;           // release counter and error flag of the single-launch bisection
  unsigned int arrived[OC_MAX_BLOCKS];      // per-CTA pass counters (arrival flags, no shared atomics)
  int steps_left, exact;                    // bisection steps still to take; next pass evaluates lmid in FP64
  double cpartial[OC_MAX_BLOCKS][OC_CAND];  // per-CTA sums of the candidates of a pass
};

__device__ __forceinline__ double oc_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ double oc_block_sum(double v) {
  __shared__ double sh[OC_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = oc_warp_sum(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (wid == 0) {
    t = lane < OC_THREADS / 32 ? sh[lane] : 0.0;
    t = oc_warp_sum(t);
  }
  __syncthreads();
  return t;
}

__global__ void oc_init_kernel(OCScratch* s, double l1, double l2, int steps) {
  for (int b = threadIdx.x; b < OC_MAX_BLOCKS; b += blockDim.x) s->arrived[b] = 0u;
  if (threadIdx.x == 0) {
    s->l1 = l1;
    s->l2 = l2;
    s->lmid = 0.5 * (l1 + l2);
    s->lmid_last = s->lmid;
    s->ticket = 0u;
    s->generation = 0u;
    s->error = 0u;
    s->steps_left = steps;
    s->exact = 0;
  }
}

// t = x sqrt(-min(dg, 0)), stored in xnew until the final step overwrites it
__global__ void oc_prepare_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ dg,
                                  double* __restrict__ t) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double g = dg[i] < 0.0 ? dg[i] : 0.0;
    t[i] = x[i] * sqrt(-g);
  }
}

__device__ __forceinline__ double oc_value(double xi, double ti, double s, double move, double xmin, double xmax) {
  const double lb = fmax(xmin, xi - move), ub = fmin(xmax, xi + move);
  return fmin(fmax(ti * s, lb), ub);
}

// One bisection step: volume of clip(t / sqrt(lmid), lb, ub); the last CTA compares it with the target and
// moves l1 or l2, exactly as OC.step does.
__global__ void __launch_bounds__(OC_THREADS) oc_step_kernel(int64_t n, const double* __restrict__ x,
                                                             const double* __restrict__ t, double target, double move,
                                                             double xmin, double xmax, OCScratch* s) {
  __shared__ double s_scale;
  const double lmid = s->lmid;
  if (threadIdx.x == 0) s_scale = 1.0 / sqrt(lmid);
  __syncthreads();
  const double sc = s_scale;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += oc_value(x[i], t[i], sc, move, xmin, xmax);
  acc = oc_block_sum(acc);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    s->partial[blockIdx.x] = acc;
    __threadfence();
    last = atomicAdd(&s->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) tot += ((volatile double*)s->partial)[b];
  tot = oc_block_sum(tot);
  if (threadIdx.x == 0) {
    if (tot - target > 0.0)
      s->l1 = lmid;
    else
      s->l2 = lmid;
    s->lmid_last = lmid;
    s->lmid = 0.5 * (s->l1 + s->l2);
    s->ticket = 0u;
  }
}

// All bisection steps in one cooperative launch (every CTA resident), with the decisions of the sequential
// bisection reproduced exactly but several taken per grid-wide exchange.  A pass evaluates the volume at the
// 31 midpoints of the next 5 bisection levels (each midpoint formed by the same repeated 0.5 (a + b) as the
// sequential loop) in FP32, from FP32 copies of x sqrt(-dg) and the bounds kept in registers; a decision is
// taken from that value only when it is farther from the target than `margin`, a bound of the FP32 error of
// the sum; the first undecided midpoint is evaluated in FP64 in the next pass, exactly as oc_step_kernel does.
// Each pass: every CTA writes its partial sums and then its pass counter; CTA 0 waits for all counters, walks
// the tree and publishes the new state through a generation counter.  No shared-address atomics; every wait is
// bounded: after OC_SPIN_LIMIT polls the kernel sets s->error and returns.  Finally xnew = the design of the
// last step, in FP64.
constexpr int OCP_PER_THREAD = 8;
constexpr unsigned OC_SPIN_LIMIT = 1u << 24;   // polls of about 0.1-0.5 us each: a few seconds at most

// Test control of the bounded waits (pmg_set_wait_test): a poll limit replacing OC_SPIN_LIMIT (0: the default)
// and a switch that makes the last CTA withhold its arrival at the grid barrier, a flag nothing else sets.
struct WaitTest {
  unsigned limit;
  unsigned withhold;
};
__device__ WaitTest g_wait_test = {0u, 0u};

__device__ __forceinline__ double oc_exact_value(double xi, double gi, double sc, double move, double xmin,
                                                 double xmax) {
  const double g = gi < 0.0 ? gi : 0.0;
  const double lb = fmax(xmin, xi - move), ub = fmin(xmax, xi + move);
  return fmin(fmax(xi * sqrt(-g) * sc, lb), ub);
}

// The same value from t = x sqrt(-min(dg, 0)) computed once (identical operations, identical result).
__device__ __forceinline__ double oc_exact_value_t(double xi, double ti, double sc, double move, double xmin,
                                                   double xmax) {
  const double lb = fmax(xmin, xi - move), ub = fmin(xmax, xi + move);
  return fmin(fmax(ti * sc, lb), ub);
}

__device__ __forceinline__ float oc_warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(OC_THREADS) oc_persistent_kernel(int64_t n, const double* __restrict__ x,
                                                                   const double* __restrict__ dg,
                                                                   double* __restrict__ xnew, double target,
                                                                   double move, double xmin, double xmax,
                                                                   double margin, OCScratch* s) {
  __shared__ double s_lm[OC_CAND];
  __shared__ float s_sc[OC_CAND];
  __shared__ double s_red[OC_CAND];
  __shared__ int s_abort, s_mode, s_depth;
  __shared__ double s_lmid;
  volatile OCScratch* vs = (volatile OCScratch*)s;
  const WaitTest wt = g_wait_test;
  const unsigned spin_limit = wt.limit ? wt.limit : OC_SPIN_LIMIT;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float t32[OCP_PER_THREAD], lo32[OCP_PER_THREAD], hi32[OCP_PER_THREAD];
  double t64[OCP_PER_THREAD], x64[OCP_PER_THREAD];   // x sqrt(-g) and x in FP64: no FP64 sqrt per pass
#pragma unroll
  for (int k = 0; k < OCP_PER_THREAD; ++k) {
    const int64_t i = i0 + k * stride;
    if (i < n) {
      const double g = dg[i] < 0.0 ? dg[i] : 0.0;
      const double xv = x[i];
      t64[k] = xv * sqrt(-g);
      x64[k] = xv;
      t32[k] = (float)t64[k];
      lo32[k] = (float)fmax(xmin, xv - move);
      hi32[k] = (float)fmin(xmax, xv + move);
    } else {
      t64[k] = x64[k] = 0.0;
      t32[k] = lo32[k] = hi32[k] = 0.f;
    }
  }
  if (threadIdx.x == 0) s_abort = 0;
  for (unsigned gen = 1;; ++gen) {
    if (threadIdx.x == 0) {
      const int left = vs->steps_left;
      s_mode = left <= 0 ? -1 : vs->exact;
      s_depth = left < OC_TREE ? left : OC_TREE;
      s_lmid = vs->lmid;
    }
    __syncthreads();
    const int mode = s_mode;
    if (mode < 0) break;
    if (mode == 0) {
      // candidate midpoints: node j of level d (j = 2^d - 1 + m) follows the bits of m from the root
      const int ncand = (1 << s_depth) - 1;
      if (threadIdx.x < ncand) {
        const int j = threadIdx.x;
        int d = 0;
        while ((2 << d) - 1 <= j) ++d;
        const int m = j - ((1 << d) - 1);
        double a = vs->l1, b = vs->l2;
        for (int q = d - 1; q >= 0; --q) {
          const double mid = 0.5 * (a + b);
          if ((m >> q) & 1) a = mid; else b = mid;
        }
        const double lm = 0.5 * (a + b);
        s_lm[j] = lm;
        s_sc[j] = (float)(1.0 / sqrt(lm));
      }
      __syncthreads();
      float acc[OC_CAND];
#pragma unroll
      for (int j = 0; j < OC_CAND; ++j) acc[j] = 0.f;
#pragma unroll
      for (int k = 0; k < OCP_PER_THREAD; ++k) {
#pragma unroll
        for (int j = 0; j < OC_CAND; ++j) acc[j] += fminf(fmaxf(t32[k] * s_sc[j], lo32[k]), hi32[k]);
      }
      // warp sums in FP32 (FP64 shuffles and adds would make the pass FP64-bound on GB300; their rounding is
      // in the margin), then the warps of the CTA in FP64, in order
      __shared__ double s_wsum[OC_THREADS / 32][OC_CAND];
#pragma unroll
      for (int j = 0; j < OC_CAND; ++j) {
        const float v = oc_warp_sum_f(acc[j]);
        if (lane == 0) s_wsum[warp][j] = (double)v;
      }
      __syncthreads();
      if (threadIdx.x < ncand) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < OC_THREADS / 32; ++w) v += s_wsum[w][threadIdx.x];
        vs->cpartial[blockIdx.x][threadIdx.x] = v;
      }
    } else {
      const double sc = 1.0 / sqrt(s_lmid);
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < OCP_PER_THREAD; ++k) {
        const int64_t i = i0 + k * stride;
        if (i < n) acc += oc_exact_value_t(x64[k], t64[k], sc, move, xmin, xmax);
      }
      acc = oc_block_sum(acc);
      if (threadIdx.x == 0) vs->partial[blockIdx.x] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (!(wt.withhold && blockIdx.x == gridDim.x - 1)) vs->arrived[blockIdx.x] = gen;
    }
    if (blockIdx.x == 0) {
      for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        unsigned polls = 0;
        while (vs->arrived[b] < gen) {
          if (++polls > spin_limit) {
            atomicExch(&s->error, 1u);
            s_abort = 1;
            break;
          }
        }
      }
      __syncthreads();
      __threadfence();
      if (mode == 0) {
        const int ncand = (1 << s_depth) - 1;
        // totals of the candidates, one warp per candidate (CTA order within the lanes' strided sums)
        for (int j = warp; j < ncand; j += OC_THREADS / 32) {
          double v = 0.0;
          for (int b = lane; b < (int)gridDim.x; b += 32) v += vs->cpartial[b][j];
          v = oc_warp_sum(v);
          if (lane == 0) s_red[j] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          double a = vs->l1, b = vs->l2;
          int j = 0, left = vs->steps_left, exact = 0;
          double lmid_last = vs->lmid_last, lmid = vs->lmid;
          for (int d = 0; d < s_depth; ++d) {
            const double lm = s_lm[j], diff = s_red[j] - target;
            if (!(fabs(diff) > margin)) {   // too close to call in FP32: evaluate this midpoint in FP64
              exact = 1;
              lmid = lm;
              break;
            }
            const bool up = diff > 0.0;
            if (up) a = lm; else b = lm;
            lmid_last = lm;
            --left;
            j = 2 * j + 1 + (up ? 1 : 0);
          }
          vs->l1 = a;
          vs->l2 = b;
          vs->lmid_last = lmid_last;
          vs->lmid = exact ? lmid : 0.5 * (a + b);
          vs->steps_left = left;
          vs->exact = exact;
          __threadfence();
          vs->generation = gen;
        }
      } else {
        double tot = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) tot += vs->partial[b];
        tot = oc_block_sum(tot);
        if (threadIdx.x == 0) {
          const double lmid = vs->lmid;
          if (tot - target > 0.0)
            vs->l1 = lmid;
          else
            vs->l2 = lmid;
          vs->lmid_last = lmid;
          vs->lmid = 0.5 * (vs->l1 + vs->l2);
          vs->steps_left = vs->steps_left - 1;
          vs->exact = 0;
          __threadfence();
          vs->generation = gen;
        }
      }
    } else if (threadIdx.x == 0) {
      unsigned polls = 0;
      while (vs->generation < gen) {
        if (++polls > spin_limit) {
          atomicExch(&s->error, 1u);
          s_abort = 1;
          break;
        }
      }
      __threadfence();
    }
    __syncthreads();
    if (s_abort) return;
  }
  const double sc = 1.0 / sqrt(vs->lmid_last);
#pragma unroll
  for (int k = 0; k < OCP_PER_THREAD; ++k) {
    const int64_t i = i0 + k * stride;
    if (i < n) xnew[i] = oc_exact_value_t(x64[k], t64[k], sc, move, xmin, xmax);
  }
}

// xnew = the design of the last bisection step (t is read from xnew and overwritten in place)
__global__ void oc_final_kernel(int64_t n, const double* __restrict__ x, double* __restrict__ xnew, double move,
                                double xmin, double xmax, const OCScratch* s) {
  const double sc = 1.0 / sqrt(s->lmid_last);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    xnew[i] = oc_value(x[i], xnew[i], sc, move, xmin, xmax);
}

}  // namespace pmg

using namespace pmg;

extern "C" {

int pmg_density_filter_rowsum(int nelx, int nely, int nelz, double radius, double* s, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !s || !(radius > 0.0)) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  density_rowsum_kernel<<<blocks_for(g.nel(), 128), 128, 0, as_stream(stream)>>>(g, radius, s);
  return check_launch();
}

int pmg_density_filter(int transpose, int nelx, int nely, int nelz, double radius, const double* s, const double* x,
                       double* y, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !s || !x || !y || x == y || !(radius > 0.0)) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const unsigned b = blocks_for(g.nel(), 128);
  if (transpose)
    density_filter_kernel<true><<<b, 128, 0, as_stream(stream)>>>(g, radius, s, x, y);
  else
    density_filter_kernel<false><<<b, 128, 0, as_stream(stream)>>>(g, radius, s, x, y);
  return check_launch();
}

int pmg_conv_filter(int nelx, int nely, int nelz, const double* w, int kx, int ky, int kz, const int32_t* padx,
                    const int32_t* pady, const int32_t* padz, const double* x, double* y, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !w || !padx || !pady || !padz || !x || !y || x == y) return PMG_BAD_ARG;
  if (kx < 1 || ky < 1 || kz < 1 || !(kx & 1) || !(ky & 1) || !(kz & 1)) return PMG_BAD_ARG;
  if (nelz == 0 && kz != 1) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  conv_filter_kernel<<<blocks_for(g.nel(), 128), 128, 0, as_stream(stream)>>>(g, w, kx, ky, kz, padx, pady, padz, x, y);
  return check_launch();
}

int pmg_conv_filter_adjoint(int nelx, int nely, int nelz, const double* w, int kx, int ky, int kz,
                            const int32_t* invx_ptr, const int32_t* invx_pos, const int32_t* invy_ptr,
                            const int32_t* invy_pos, const int32_t* invz_ptr, const int32_t* invz_pos,
                            const double* d, double* y, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !w || !invx_ptr || !invx_pos || !invy_ptr || !invy_pos || !invz_ptr ||
      !invz_pos || !d || !y || d == y)
    return PMG_BAD_ARG;
  if (kx < 1 || ky < 1 || kz < 1 || !(kx & 1) || !(ky & 1) || !(kz & 1)) return PMG_BAD_ARG;
  if (nelz == 0 && kz != 1) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  conv_filter_adjoint_kernel<<<blocks_for(g.nel(), 128), 128, 0, as_stream(stream)>>>(
      g, w, kx, ky, kz, invx_ptr, invx_pos, invy_ptr, invy_pos, invz_ptr, invz_pos, d, y);
  return check_launch();
}

int pmg_simp(int64_t n, double xmin, double penal, const double* x, double* y, void* y32, void* stream) {
  if (n < 0 || !x || (!y && !y32)) return PMG_BAD_ARG;
  if (n == 0) return PMG_OK;
  simp_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(n, xmin, penal, x, y, (float*)y32);
  return check_launch();
}

int pmg_simp_backward(int64_t n, double xmin, double penal, const double* x, const double* dy, double* dx,
                      void* stream) {
  if (n < 0 || !x || !dy || !dx) return PMG_BAD_ARG;
  if (n == 0) return PMG_OK;
  simp_backward_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(n, xmin, penal, x, dy, dx);
  return check_launch();
}

int pmg_sens_contract(int nelx, int nely, int nelz, const double* K0_host, const uint8_t* bcmask, const double* u,
                      const double* v, double alpha, int accumulate, double* dx, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !K0_host || !u || !v || !dx) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const unsigned b = blocks_for(g.nel(), 128);
  if (g.dim() == 3)
    sens_kernel<3><<<b, 128, 0, as_stream(stream)>>>(g, make_elem_mat<double, 24>(K0_host), bcmask, u, v, alpha,
                                                     accumulate, dx);
  else
    sens_kernel<2><<<b, 128, 0, as_stream(stream)>>>(g, make_elem_mat<double, 8>(K0_host), bcmask, u, v, alpha,
                                                     accumulate, dx);
  return check_launch();
}

int pmg_sens_contract_mixed(int nelx, int nely, int nelz, const double* K0_host, const uint8_t* bcmask,
                            const double* u, const double* v, double alpha, int accumulate, double* dx,
                            void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !K0_host || !u || !v || !dx) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const unsigned b = blocks_for(g.nel(), 128);
  if (g.dim() == 3) {
    // z chunks: about two CTAs per SM in one wave, at least 4 layers per chunk
    const int tx = (g.nx + SENS_TX - 1) / SENS_TX, ty = (g.ny + SENS_TY - 1) / SENS_TY;
    int nzc = std::max(1, std::min(g.nz / 4, (2 * sm_count() + tx * ty - 1) / (tx * ty)));
    const int zchunk = (g.nz + nzc - 1) / nzc;
    nzc = (g.nz + zchunk - 1) / zchunk;
    sens_mixed_tiled_kernel<<<dim3(tx, ty, nzc), SENS_TX * SENS_TY, 0, as_stream(stream)>>>(
        g, make_elem_mat<float, 24>(K0_host), bcmask, u, v, alpha, accumulate, zchunk, dx);
  } else
    sens_mixed_kernel<2><<<b, 128, 0, as_stream(stream)>>>(g, make_elem_mat<float, 8>(K0_host), bcmask, u, v, alpha,
                                                           accumulate, dx);
  return check_launch();
}

size_t pmg_oc_scratch_bytes(void) { return sizeof(OCScratch); }

int pmg_set_wait_test(unsigned polls, int withhold_arrival) {
  const WaitTest wt = {polls, withhold_arrival ? 1u : 0u};
  cudaError_t e = cudaMemcpyToSymbol(g_wait_test, &wt, sizeof(wt));
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return PMG_OK;
}

int pmg_oc_status(const void* scratch) {
  if (!scratch) return PMG_BAD_ARG;
  unsigned err = 0;
  cudaError_t e = cudaMemcpy(&err, &((const OCScratch*)scratch)->error, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return err ? PMG_TIMEOUT : PMG_OK;
}

int pmg_oc_status_async(const void* scratch, unsigned* status, void* stream) {
  if (!scratch || !status) return PMG_BAD_ARG;
  cudaError_t e = cudaMemcpyAsync(status, &((const OCScratch*)scratch)->error, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                  as_stream(stream));
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return PMG_OK;
}

int pmg_oc_update(int64_t n, const double* x, const double* dg, double* xnew, double volfrac, double move, double xmin,
                  double xmax, double l1, double l2, double l1l2tol, void* scratch, void* stream) {
  if (n <= 0 || !x || !dg || !xnew || !scratch || !(l1l2tol > 0.0) || !(l2 >= l1)) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  OCScratch* s = (OCScratch*)scratch;
  int64_t nb = (n + OC_THREADS * 8 - 1) / (OC_THREADS * 8);
  if (nb > 2 * 152) nb = 2 * 152;
  if (nb < 1) nb = 1;
  if (x == xnew || dg == xnew) return PMG_BAD_ARG;
  // the interval halves every step, so the step count is known on the host: same loop as OC.step
  double a = l1, b = l2;
  const double target = volfrac * (double)n;
  int steps = 0;
  while (b - a > l1l2tol) {
    a = 0.5 * (a + b);  // only the interval width matters for the count
    if (++steps > 200) return PMG_BAD_ARG;
  }
  oc_init_kernel<<<1, 256, 0, st>>>(s, l1, l2, steps);
  // single cooperative launch when every element fits in the registers of co-resident CTAs
  static int coop_blocks[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    if (coop_blocks[dev] == 0) {
      int sms = 0, per_sm = 0, coop = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, oc_persistent_kernel, OC_THREADS, 0);
      coop_blocks[dev] = coop ? std::min(sms * per_sm, OC_MAX_BLOCKS) : -1;
    }
    const int cb = coop_blocks[dev];
    if (cb > 0 && n <= (int64_t)cb * OC_THREADS * OCP_PER_THREAD) {
      const int grid = cb;   // all co-resident slots: the fewest elements per thread
      // bound of the FP32 error of a candidate volume: per element 3 roundings of a value up to M, the FP32
      // sum of at most OCP_PER_THREAD values per thread (each addition off by <= u32 * OCP_PER_THREAD * M, at
      // most one addition per element), and the 5 levels of the FP32 warp sum (each level off by u32 times the
      // partial sums, at most 32 * OCP_PER_THREAD * M per lane pair: <= 5 u32 M per element in total); the
      // sums over warps and CTAs are FP64; doubled for safety
      const double M = std::max({1.0, std::fabs(xmin), std::fabs(xmax)});
      const double u32 = std::ldexp(1.0, -24);
      const double margin = 2.0 * (3.0 + OCP_PER_THREAD + 5.0) * (double)n * u32 * M;
      void* args[] = {(void*)&n, (void*)&x, (void*)&dg, (void*)&xnew, (void*)&target, (void*)&move,
                      (void*)&xmin, (void*)&xmax, (void*)&margin, (void*)&s};
      cudaError_t e = cudaLaunchCooperativeKernel((const void*)oc_persistent_kernel, dim3(grid), dim3(OC_THREADS),
                                                  args, 0, st);
      if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return PMG_CUDA_ERR;
      }
      return check_launch();
    }
  }
  oc_prepare_kernel<<<(unsigned)nb, OC_THREADS, 0, st>>>(n, x, dg, xnew);
  for (int k = 0; k < steps; ++k)
    oc_step_kernel<<<(unsigned)nb, OC_THREADS, 0, st>>>(n, x, xnew, target, move, xmin, xmax, s);
  oc_final_kernel<<<(unsigned)nb, OC_THREADS, 0, st>>>(n, x, xnew, move, xmin, xmax, s);
  return check_launch();
}

}  // extern "C"
