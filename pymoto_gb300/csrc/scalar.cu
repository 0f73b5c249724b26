// One-component operators: one dof per node (thermal / Poisson problems and the scalar mass matrix of
// pymoto/modules/assembly.py:466-560, AssemblePoisson and AssembleMass with ndof = 1).
//
// Storage: the full node stencil S[o][n] with o = (dz + 1) 9 + (dy + 1) 3 + (dx + 1) (27 offsets in 3D, 9 in 2D),
// zero for neighbours outside the grid.  Assembly sums x_e P0 over the elements a node pair shares; Dirichlet rows
// and columns (bit 0 of the node's mask byte) hold bcdiag on the diagonal only, and the constant diagonal of
// add_constant is added to every row (pymoto/modules/assembly.py:245-296).  The Galerkin coarse operator R^T A R is
// formed stencil to stencil with the trilinear (bilinear) prolongation of GeometricMultigrid
// (pymoto/solvers/iterative.py:124-256).  Every sum has a fixed order: deterministic results.
#include <type_traits>

#include "common.cuh"

namespace pmg {
namespace {

template <int DIM>
struct SC {
  static constexpr int NN = 1 << DIM;                 // nodes per element
  static constexpr int NOFF = DIM == 3 ? 27 : 9;      // stencil offsets
  static constexpr int CENTER = NOFF / 2;
};

__device__ __forceinline__ double sc_tw(int a) { return a == 0 ? 1.0 : 0.5; }

template <typename T, int DIM>
__global__ void scalar_stencil_kernel(Grid g, const double* __restrict__ xe, ElemMat<double, SC<DIM>::NN> P0,
                                      const uint8_t* __restrict__ bcmask, double bcdiag,
                                      const double* __restrict__ cdiag, T* __restrict__ S) {
  constexpr int NOFF = SC<DIM>::NOFF, CENTER = SC<DIM>::CENTER, NN = SC<DIM>::NN;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  const bool nfix = bcmask && (bcmask[n] & 1u);
  for (int o = 0; o < NOFF; ++o) {
    int dx, dy, dz;
    stencil_offset<DIM>(o, dx, dy, dz);
    const int mi = i + dx, mj = j + dy, mk = k + dz;
    double v = 0.0;
    if (mi >= 0 && mi <= g.nx && mj >= 0 && mj <= g.ny && mk >= 0 && mk <= g.nz) {
      const int64_t m = node_id(g, mi, mj, mk);
      const bool mfix = bcmask && (bcmask[m] & 1u);
      if (nfix) {
        if (o == CENTER) v = bcdiag;
      } else if (!mfix) {
        double acc = 0.0;
        // elements (i - 1 + ex, j - 1 + ey, k - 1 + ez) hold node n; those that also hold m add x_e P0[n][m]
        for (int ez = 0; ez < (DIM == 3 ? 2 : 1); ++ez)
          for (int ey = 0; ey < 2; ++ey)
            for (int ex = 0; ex < 2; ++ex) {
              const int ei = i - 1 + ex, ej = j - 1 + ey, ek = DIM == 3 ? k - 1 + ez : 0;
              if (ei < 0 || ei >= g.nx || ej < 0 || ej >= g.ny || (DIM == 3 && (ek < 0 || ek >= g.nz))) continue;
              const int lmx = mi - ei, lmy = mj - ej, lmz = DIM == 3 ? mk - ek : 0;
              if (lmx < 0 || lmx > 1 || lmy < 0 || lmy > 1 || lmz < 0 || lmz > 1) continue;
              const int ln = (i - ei) + 2 * (j - ej) + 4 * (DIM == 3 ? k - ek : 0);
              const int lm = lmx + 2 * lmy + 4 * lmz;
              acc += xe[elem_id(g, ei, ej, ek)] * P0.v[ln * NN + lm];
            }
        v = acc;
      }
      if (o == CENTER && cdiag) v += cdiag[n];
    }
    S[(int64_t)o * nn + n] = (T)v;
  }
}

// y = S u (mode 0), b - S u (1), u + w (b - S u) / diag (2)
template <typename T, int DIM, int MODE>
__global__ void scalar_apply_kernel(Grid g, const T* __restrict__ S, const T* __restrict__ u, const T* __restrict__ b,
                                    const T* __restrict__ diag, T w, T* __restrict__ y) {
  constexpr int NOFF = SC<DIM>::NOFF;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  T acc = T(0);
#pragma unroll
  for (int o = 0; o < NOFF; ++o) {
    int dx, dy, dz;
    stencil_offset<DIM>(o, dx, dy, dz);
    // out-of-grid neighbours have zero coefficients: their value is read at a clamped index
    const int mi = min(max(i + dx, 0), g.nx), mj = min(max(j + dy, 0), g.ny), mk = min(max(k + dz, 0), g.nz);
    acc = fma(S[(int64_t)o * nn + n], u[node_id(g, mi, mj, mk)], acc);
  }
  if (MODE == 0) {
    y[n] = acc;
  } else if (MODE == 1) {
    y[n] = b[n] - acc;
  } else {
    y[n] = u[n] + w * ((b[n] - acc) / diag[n]);
  }
}

// rc = R^T rf over the fine grid gf
template <typename T, int DIM>
__global__ void scalar_restrict_kernel(Grid gf, const T* __restrict__ rf, T* __restrict__ rc) {
  const Grid gc = gf.coarse();
  const int64_t N = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (N >= gc.nnodes()) return;
  int I, J, K;
  node_ijk(gc, N, I, J, K);
  T acc = T(0);
  for (int c = (DIM == 3 ? -1 : 0); c <= (DIM == 3 ? 1 : 0); ++c)
    for (int bb = -1; bb <= 1; ++bb)
      for (int a = -1; a <= 1; ++a) {
        const int i = 2 * I + a, j = 2 * J + bb, k = 2 * K + c;
        if (i < 0 || i > gf.nx || j < 0 || j > gf.ny || k < 0 || k > gf.nz) continue;
        acc = fma((T)(sc_tw(a) * sc_tw(bb) * sc_tw(c)), rf[node_id(gf, i, j, k)], acc);
      }
  rc[N] = acc;
}

// uf += R uc over the fine grid gf
template <typename T, int DIM>
__global__ void scalar_prolong_add_kernel(Grid gf, const T* __restrict__ uc, T* __restrict__ uf) {
  const Grid gc = gf.coarse();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= gf.nnodes()) return;
  int i, j, k;
  node_ijk(gf, n, i, j, k);
  T acc = T(0);
  for (int pz = 0; pz <= (DIM == 3 ? (k & 1) : 0); ++pz)
    for (int py = 0; py <= (j & 1); ++py)
      for (int px = 0; px <= (i & 1); ++px) {
        const T wgt = (T)(((i & 1) ? 0.5 : 1.0) * ((j & 1) ? 0.5 : 1.0) * ((DIM == 3 && (k & 1)) ? 0.5 : 1.0));
        acc = fma(wgt, uc[node_id(gc, (i >> 1) + px, (j >> 1) + py, (k >> 1) + pz)], acc);
      }
  uf[n] += acc;
}

// Coarse offsets q (per axis, from -1 to 1) whose prolongation column holds the fine offset e = a + d (-2 .. 2)
// from 2N: e / 2 with weight 1 for even e, (e - 1) / 2 and (e + 1) / 2 with weight 1/2 each for odd e.
__host__ __device__ constexpr int sc_lo(int e) { return (e & 1) ? (e - 1) / 2 : e / 2; }
__host__ __device__ constexpr int sc_cnt(int e) { return (e & 1) ? 2 : 1; }
__host__ __device__ constexpr double sc_wt(int e) { return (e & 1) ? 0.5 : 1.0; }

// Sc = R^T Sf R: per coarse node N, the fine nodes n = 2N + a of its prolongation column (weight w(a)), each of
// their stencil entries (n, n + d), and the coarse nodes N + q whose column holds n + d: Sc(N, q) += w(a) Sf(n, d)
// w'(a + d, q).  Both loops are unrolled, so every accumulator index is a compile-time constant (the sums stay in
// registers).  R^T S R is symmetric, so only the centre and the forward offsets q >= CENTER are summed here (half
// the FMAs, and no load of an entry that reaches only backward offsets); scalar_mirror_kernel copies the backward
// ones from the neighbours.  FP64 operators accumulate in FP64, FP32 operators in FP32 (their hierarchy is a
// preconditioner).
template <typename T, int DIM>
__global__ void __launch_bounds__(128) scalar_galerkin_kernel(Grid gf, const T* __restrict__ Sf, T* __restrict__ Sc) {
  constexpr int NOFF = SC<DIM>::NOFF, CENTER = SC<DIM>::CENTER;
  const Grid gc = gf.coarse();
  const int64_t nnf = gf.nnodes(), nnc = gc.nnodes();
  const int64_t N = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (N >= nnc) return;
  int I, J, K;
  node_ijk(gc, N, I, J, K);
  T acc[NOFF];
#pragma unroll
  for (int q = 0; q < NOFF; ++q) acc[q] = T(0);
#pragma unroll
  for (int ia = 0; ia < NOFF; ++ia) {
    int ax, ay, az;
    stencil_offset<DIM>(ia, ax, ay, az);
    const int i = 2 * I + ax, j = 2 * J + ay, k = 2 * K + az;
    const bool in = i >= 0 && i <= gf.nx && j >= 0 && j <= gf.ny && k >= 0 && k <= gf.nz;
    const int64_t n = in ? node_id(gf, i, j, k) : 0;
    const T wn = (T)(sc_tw(ax) * sc_tw(ay) * sc_tw(az));
#pragma unroll
    for (int o = 0; o < NOFF; ++o) {
      int dx, dy, dz;
      stencil_offset<DIM>(o, dx, dy, dz);
      const int ex = ax + dx, ey = ay + dy, ez = az + dz;
      // the largest target offset of this entry; an entry that reaches only backward offsets is not loaded
      const int qmax = DIM == 3 ? (sc_lo(ez) + sc_cnt(ez)) * 9 + (sc_lo(ey) + sc_cnt(ey)) * 3 + (sc_lo(ex) + sc_cnt(ex))
                                : (sc_lo(ey) + sc_cnt(ey)) * 3 + (sc_lo(ex) + sc_cnt(ex));
      if (qmax < CENTER) continue;
      // coefficients towards fine nodes outside the grid are zero, so only n itself needs the bounds test
      const T s = in ? wn * Sf[(int64_t)o * nnf + n] : T(0);
#pragma unroll
      for (int qz = 0; qz < sc_cnt(ez); ++qz)
#pragma unroll
        for (int qy = 0; qy < sc_cnt(ey); ++qy)
#pragma unroll
          for (int qx = 0; qx < sc_cnt(ex); ++qx) {
            const int Ox = sc_lo(ex) + qx, Oy = sc_lo(ey) + qy, Oz = sc_lo(ez) + qz;
            const int q = DIM == 3 ? (Oz + 1) * 9 + (Oy + 1) * 3 + (Ox + 1) : (Oy + 1) * 3 + (Ox + 1);
            if (q >= CENTER) acc[q] = fma((T)(sc_wt(ex) * sc_wt(ey) * sc_wt(ez)), s, acc[q]);
          }
    }
  }
  // coefficients towards coarse nodes outside the grid are zero by construction (no fine node there)
#pragma unroll
  for (int q = CENTER; q < NOFF; ++q) Sc[(int64_t)q * nnc + N] = acc[q];
}

// Backward offsets of a symmetric stencil from its forward ones: S(N, q) = S(N + off(q), NOFF - 1 - q) for
// q < CENTER, zero towards nodes outside the grid.
template <typename T, int DIM>
__global__ void scalar_mirror_kernel(Grid g, T* __restrict__ S) {
  constexpr int NOFF = SC<DIM>::NOFF, CENTER = SC<DIM>::CENTER;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
#pragma unroll
  for (int q = 0; q < CENTER; ++q) {
    int dx, dy, dz;
    stencil_offset<DIM>(q, dx, dy, dz);
    const int mi = i + dx, mj = j + dy, mk = k + dz;
    const bool in = mi >= 0 && mi <= g.nx && mj >= 0 && mj <= g.ny && mk >= 0 && mk <= g.nz;
    S[(int64_t)q * nn + n] = in ? S[(int64_t)(NOFF - 1 - q) * nn + node_id(g, mi, mj, mk)] : T(0);
  }
}

// A (n x n FP64, zero-filled before) gets the stencil entries
template <typename T, int DIM>
__global__ void scalar_to_dense_kernel(Grid g, const T* __restrict__ S, double* __restrict__ A) {
  constexpr int NOFF = SC<DIM>::NOFF;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  for (int o = 0; o < NOFF; ++o) {
    int dx, dy, dz;
    stencil_offset<DIM>(o, dx, dy, dz);
    const int mi = i + dx, mj = j + dy, mk = k + dz;
    if (mi < 0 || mi > g.nx || mj < 0 || mj > g.ny || mk < 0 || mk > g.nz) continue;
    A[n * nn + node_id(g, mi, mj, mk)] = (double)S[(int64_t)o * nn + n];
  }
}

// d = sum_o |S(n, o)|: the l1 row sums
template <typename T, int DIM>
__global__ void scalar_rowabs_kernel(Grid g, const T* __restrict__ S, T* __restrict__ d) {
  constexpr int NOFF = SC<DIM>::NOFF;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  T acc = T(0);
#pragma unroll
  for (int o = 0; o < NOFF; ++o) acc += abs(S[(int64_t)o * nn + n]);
  d[n] = acc;
}

// dx_e (+)= alpha u_e^T P0 v_e, Dirichlet nodes of u and v taken as zero
template <int DIM>
__global__ void scalar_sens_kernel(Grid g, ElemMat<double, SC<DIM>::NN> P0, const uint8_t* __restrict__ bcmask,
                                   const double* __restrict__ u, const double* __restrict__ v, double alpha,
                                   int accumulate, double* __restrict__ dx) {
  constexpr int NN = SC<DIM>::NN;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  const int i = (int)(e % g.nx), j = (int)((e / g.nx) % g.ny), k = (int)(e / ((int64_t)g.nx * g.ny));
  double ue[NN], ve[NN];
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    const int64_t n = node_id(g, i + (a & 1), j + ((a >> 1) & 1), k + (a >> 2));
    const bool fixed = bcmask && (bcmask[n] & 1u);
    ue[a] = fixed ? 0.0 : u[n];
    ve[a] = fixed ? 0.0 : v[n];
  }
  double acc = 0.0;
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    double t = 0.0;
#pragma unroll
    for (int b = 0; b < NN; ++b) t = fma(P0.v[a * NN + b], ve[b], t);
    acc = fma(ue[a], t, acc);
  }
  dx[e] = (accumulate ? dx[e] : 0.0) + alpha * acc;
}

template <int NN>
ElemMat<double, NN> host_mat(const double* P0) {
  ElemMat<double, NN> m;
  for (int q = 0; q < NN * NN; ++q) m.v[q] = P0[q];
  return m;
}

bool scalar_grid(int nx, int ny, int nz) { return grid_ok(nx, ny, nz); }

}  // namespace
}  // namespace pmg

using namespace pmg;

// Runs f(T{}, std::integral_constant<int, DIM>{}) for the dtype and the dimension of the grid, then checks the launch.
template <typename F>
static int scalar_dispatch(int dtype, int nz, F&& f) {
  if (dtype == PMG_F64 && nz > 0)
    f(double{}, std::integral_constant<int, 3>{});
  else if (dtype == PMG_F64)
    f(double{}, std::integral_constant<int, 2>{});
  else if (dtype == PMG_F32 && nz > 0)
    f(float{}, std::integral_constant<int, 3>{});
  else if (dtype == PMG_F32)
    f(float{}, std::integral_constant<int, 2>{});
  else
    return PMG_BAD_ARG;
  return check_launch();
}

#define PMG_SCALAR_TYPES      \
  using T = decltype(t_);     \
  constexpr int DIM = decltype(dim_)::value

extern "C" {

int pmg_scalar_stencil(int dtype, int nelx, int nely, int nelz, const double* xe, const double* P0_host,
                       const uint8_t* bcmask, double bcdiag, const double* cdiag, void* S, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !xe || !P0_host || !S) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.nnodes(), 256);
  cudaStream_t st = as_stream(stream);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    scalar_stencil_kernel<T, DIM><<<blocks, 256, 0, st>>>(g, xe, host_mat<SC<DIM>::NN>(P0_host), bcmask, bcdiag,
                                                          cdiag, (T*)S);
  });
}

int pmg_scalar_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* S, const void* u, const void* b,
                     const void* diag, double omega, void* y, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !S || !u || !y || y == u || mode < 0 || mode > 2) return PMG_BAD_ARG;
  if (mode >= PMG_APPLY_RESIDUAL && !b) return PMG_BAD_ARG;
  if (mode == PMG_APPLY_JACOBI && !diag) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.nnodes(), 256);
  cudaStream_t st = as_stream(stream);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    const T* S_ = (const T*)S;
    const T* u_ = (const T*)u;
    const T* b_ = (const T*)b;
    const T* d_ = (const T*)diag;
    T* y_ = (T*)y;
    if (mode == PMG_APPLY_MATVEC)
      scalar_apply_kernel<T, DIM, 0><<<blocks, 256, 0, st>>>(g, S_, u_, b_, d_, (T)omega, y_);
    else if (mode == PMG_APPLY_RESIDUAL)
      scalar_apply_kernel<T, DIM, 1><<<blocks, 256, 0, st>>>(g, S_, u_, b_, d_, (T)omega, y_);
    else
      scalar_apply_kernel<T, DIM, 2><<<blocks, 256, 0, st>>>(g, S_, u_, b_, d_, (T)omega, y_);
  });
}

static bool even(int nx, int ny, int nz) { return nx % 2 == 0 && ny % 2 == 0 && nz % 2 == 0 && nx >= 2 && ny >= 2; }

int pmg_scalar_restrict(int dtype, int nelx, int nely, int nelz, const void* rf, void* rc, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !even(nelx, nely, nelz) || !rf || !rc) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.coarse().nnodes(), 256);
  cudaStream_t st = as_stream(stream);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    scalar_restrict_kernel<T, DIM><<<blocks, 256, 0, st>>>(g, (const T*)rf, (T*)rc);
  });
}

int pmg_scalar_prolong_add(int dtype, int nelx, int nely, int nelz, const void* uc, void* uf, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !even(nelx, nely, nelz) || !uc || !uf) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.nnodes(), 256);
  cudaStream_t st = as_stream(stream);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    scalar_prolong_add_kernel<T, DIM><<<blocks, 256, 0, st>>>(g, (const T*)uc, (T*)uf);
  });
}

int pmg_scalar_galerkin(int dtype, int nelx, int nely, int nelz, const void* Sf, void* Sc, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !even(nelx, nely, nelz) || !Sf || !Sc) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.coarse().nnodes(), 128);
  cudaStream_t st = as_stream(stream);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    scalar_galerkin_kernel<T, DIM><<<blocks, 128, 0, st>>>(g, (const T*)Sf, (T*)Sc);
    scalar_mirror_kernel<T, DIM><<<blocks_for(g.coarse().nnodes(), 256), 256, 0, st>>>(g.coarse(), (T*)Sc);
  });
}

int pmg_scalar_to_dense(int dtype, int nelx, int nely, int nelz, const void* S, double* A, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !S || !A) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const int64_t nn = g.nnodes();
  if (nn > 65536) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(A, 0, (size_t)nn * nn * sizeof(double), st) != cudaSuccess) return check_launch();
  const unsigned blocks = blocks_for(nn, 256);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    scalar_to_dense_kernel<T, DIM><<<blocks, 256, 0, st>>>(g, (const T*)S, (double*)A);
  });
}

int pmg_scalar_rowabs(int dtype, int nelx, int nely, int nelz, const void* S, void* d, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !S || !d) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.nnodes(), 256);
  cudaStream_t st = as_stream(stream);
  return scalar_dispatch(dtype, nelz, [&](auto t_, auto dim_) {
    PMG_SCALAR_TYPES;
    scalar_rowabs_kernel<T, DIM><<<blocks, 256, 0, st>>>(g, (const T*)S, (T*)d);
  });
}

int pmg_scalar_sens(int nelx, int nely, int nelz, const double* P0_host, const uint8_t* bcmask, const double* u,
                    const double* v, double alpha, int accumulate, double* dx, void* stream) {
  if (!scalar_grid(nelx, nely, nelz) || !P0_host || !u || !v || !dx) return PMG_BAD_ARG;
  const Grid g{nelx, nely, nelz};
  const unsigned blocks = blocks_for(g.nel(), 256);
  cudaStream_t st = as_stream(stream);
  if (nelz > 0)
    scalar_sens_kernel<3><<<blocks, 256, 0, st>>>(g, host_mat<8>(P0_host), bcmask, u, v, alpha, accumulate, dx);
  else
    scalar_sens_kernel<2><<<blocks, 256, 0, st>>>(g, host_mat<4>(P0_host), bcmask, u, v, alpha, accumulate, dx);
  return check_launch();
}

}  // extern "C"
