// Stiffness operators of the multigrid hierarchy.
//
//  level 0: matrix-free K(x) u = sum_e x_e K0 u_e with Dirichlet rows/cols (node-centric gather: every
//           thread owns one node, reads the 3^dim neighbourhood of u once into registers and sums the
//           2^dim element contributions; no atomics, deterministic).
//  level>0: assembled node stencils (3^dim blocks of dim x dim per node, structure-of-arrays).
//  transfers: trilinear restriction / prolongation as gathers.
//  Galerkin: coarse element matrices E_C = sum_c M_c^T E_c M_c by sum factorisation.
#include <cstdio>

#include <algorithm>
#include <atomic>

#include <type_traits>

#include "common.cuh"

namespace pmg {

// ------------------------------------------------------------------------------------------ level 0
// MODE 0: y = K u;  1: y = b - K u;  2: y = u + w * ((b - K u) / diag)
template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(128) ebe_apply_kernel(Grid g, const T* __restrict__ xe, ElemMat<T, Traits<DIM>::NDE> K0,
                                                        const uint8_t* __restrict__ bcmask, T bcdiag,
                                                        const T* __restrict__ u, const T* __restrict__ b,
                                                        const T* __restrict__ diag, T w, T* __restrict__ y,
                                                        const T* __restrict__ cdiag) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int KZ = DIM == 3 ? 3 : 1;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.nnodes()) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);

  // neighbourhood of u (Dirichlet columns zeroed, outside the grid zero)
  T un[KZ * 9][DIM];
#pragma unroll
  for (int dz = 0; dz < KZ; ++dz)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int ii = i + dx - 1, jj = j + dy - 1, kk = k + (DIM == 3 ? dz - 1 : 0);
        const bool in = ii >= 0 && ii <= g.nx && jj >= 0 && jj <= g.ny && kk >= 0 && kk <= g.nz;
        const int o = (dz * 3 + dy) * 3 + dx;
        if (in) {
          const int64_t m = node_id(g, ii, jj, kk);
          const uint8_t msk = bcmask ? bcmask[m] : 0;
#pragma unroll
          for (int c = 0; c < DIM; ++c) un[o][c] = (msk >> c) & 1 ? T(0) : u[m * DIM + c];
        } else {
#pragma unroll
          for (int c = 0; c < DIM; ++c) un[o][c] = T(0);
        }
      }

  T acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = T(0);

  // the 2^dim elements around the node; element offset (ox,oy,oz) has its min corner at node - 1 + o
#pragma unroll
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int ei = i - 1 + ox, ej = j - 1 + oy, ek = (DIM == 3) ? k - 1 + oz : 0;
        const bool ein = ei >= 0 && ei < g.nx && ej >= 0 && ej < g.ny && ek >= 0 && ek < g.ez();
        if (!ein) continue;
        const T x = xe[elem_id(g, ei, ej, ek)];
        constexpr int dummy = 0;
        (void)dummy;
        const int ln = (1 - ox) + 2 * (1 - oy) + 4 * (DIM == 3 ? (1 - oz) : 0);  // local index of this node
        T t[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) t[d] = T(0);
#pragma unroll
        for (int lb = 0; lb < NN; ++lb) {
          const int bx = lb & 1, by = (lb >> 1) & 1, bz = (lb >> 2) & 1;
          const int o = ((DIM == 3 ? (oz + bz) : 0) * 3 + (oy + by)) * 3 + (ox + bx);
#pragma unroll
          for (int d = 0; d < DIM; ++d)
#pragma unroll
            for (int c = 0; c < DIM; ++c) t[d] = fma(K0.v[(ln * DIM + d) * NDE + lb * DIM + c], un[o][c], t[d]);
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = fma(x, t[d], acc[d]);
      }

  const uint8_t mymask = bcmask ? bcmask[n] : 0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const int64_t q = n * DIM + d;
    T Au = ((mymask >> d) & 1) ? bcdiag * u[q] : acc[d];
    if (cdiag) Au += cdiag[q] * u[q];        // constant diagonal term (AssembleStiffness add_constant)
    if (MODE == 0) {
      y[q] = Au;
    } else if (MODE == 1) {
      y[q] = b[q] - Au;
    } else {
      y[q] = u[q] + w * ((b[q] - Au) / diag[q]);
    }
  }
}

// 3D tiled variant: a CTA owns a BX x BY x BZ brick of nodes.  It stages the u of the brick plus a one-node
// halo in shared memory (Dirichlet components and nodes outside the grid stored as zero) and the x_e of
// the (BX+1)(BY+1)(BZ+1) surrounding elements (zero outside the grid), so every thread reads its 27
// neighbours and 8 elements at constant shared-memory offsets with no bounds or mask logic.
constexpr int TBX = 32, TBY = 4, TBZ = 2;

// Shared-memory loads the compiler may not re-issue at every use: the 81 neighbour values are read once
// and stay in registers for the 600 FMAs (otherwise it rematerialises a shared load per FMA).
__device__ __forceinline__ float lds_keep(const float* p) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"((unsigned)__cvta_generic_to_shared(p)));
  return v;
}
__device__ __forceinline__ double lds_keep(const double* p) {
  double v;
  asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"((unsigned)__cvta_generic_to_shared(p)));
  return v;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(TBX * TBY * TBZ) ebe_apply_tiled_kernel(Grid g, const T* __restrict__ xe,
                                                                         ElemMat<T, 24> K0,
                                                                         const uint8_t* __restrict__ bcmask, T bcdiag,
                                                                         const T* __restrict__ u, const T* __restrict__ b,
                                                                         const T* __restrict__ diag, T w,
                                                                         T* __restrict__ y,
                                                                         const T* __restrict__ cdiag) {
  constexpr int UX = TBX + 2, UY = TBY + 2, UZ = TBZ + 2;   // node tile with halo
  constexpr int EX = TBX + 1, EY = TBY + 1, EZ = TBZ + 1;   // element tile
  constexpr int NT = TBX * TBY * TBZ;
  __shared__ T su[UZ][UY][UX][3];
  __shared__ T sx[EZ][EY][EX];
  const int i0 = blockIdx.x * TBX, j0 = blockIdx.y * TBY, k0 = blockIdx.z * TBZ;
  const int tid = threadIdx.x + TBX * (threadIdx.y + TBY * threadIdx.z);
  // stage u (coalesced along x: consecutive q -> consecutive component, then node)
  for (int q = tid; q < UX * UY * UZ * 3; q += NT) {
    const int c = q % 3, t = q / 3;
    const int lx = t % UX, ly = (t / UX) % UY, lz = t / (UX * UY);
    const int gi = i0 - 1 + lx, gj = j0 - 1 + ly, gk = k0 - 1 + lz;
    T v = T(0);
    if (gi >= 0 && gi <= g.nx && gj >= 0 && gj <= g.ny && gk >= 0 && gk <= g.nz) {
      const int64_t m = node_id(g, gi, gj, gk);
      const uint8_t msk = bcmask ? bcmask[m] : 0;
      if (!((msk >> c) & 1)) v = u[m * 3 + c];
    }
    (&su[0][0][0][0])[q] = v;
  }
  for (int q = tid; q < EX * EY * EZ; q += NT) {
    const int lx = q % EX, ly = (q / EX) % EY, lz = q / (EX * EY);
    const int gi = i0 - 1 + lx, gj = j0 - 1 + ly, gk = k0 - 1 + lz;
    T v = T(0);
    if (gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny && gk >= 0 && gk < g.nz) v = xe[elem_id(g, gi, gj, gk)];
    (&sx[0][0][0])[q] = v;
  }
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
  const int i = i0 + tx, j = j0 + ty, k = k0 + tz;
  if (i > g.nx || j > g.ny || k > g.nz) return;
  T un[27][3];
#pragma unroll
  for (int dz = 0; dz < 3; ++dz)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dx = 0; dx < 3; ++dx)
#pragma unroll
        for (int c = 0; c < 3; ++c) un[(dz * 3 + dy) * 3 + dx][c] = lds_keep(&su[tz + dz][ty + dy][tx + dx][c]);
  T acc[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int oz = 0; oz < 2; ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const T x = lds_keep(&sx[tz + oz][ty + oy][tx + ox]);
        const int ln = (1 - ox) + 2 * (1 - oy) + 4 * (1 - oz);
        T t[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int lb = 0; lb < 8; ++lb) {
          const int o = ((oz + ((lb >> 2) & 1)) * 3 + (oy + ((lb >> 1) & 1))) * 3 + (ox + (lb & 1));
#pragma unroll
          for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int c = 0; c < 3; ++c) t[d] = fma(K0.v[(ln * 3 + d) * 24 + lb * 3 + c], un[o][c], t[d]);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) acc[d] = fma(x, t[d], acc[d]);
      }
  const int64_t n = node_id(g, i, j, k);
  const uint8_t mymask = bcmask ? bcmask[n] : 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int64_t q = n * 3 + d;
    const T uq = u[q];
    T Au = ((mymask >> d) & 1) ? bcdiag * uq : acc[d];
    if (cdiag) Au += cdiag[q] * uq;
    if (MODE == 0) {
      y[q] = Au;
    } else if (MODE == 1) {
      y[q] = b[q] - Au;
    } else {
      y[q] = uq + w * ((b[q] - Au) / diag[q]);
    }
  }
}

template <typename T, int DIM>
__global__ void ebe_diag_kernel(Grid g, const T* __restrict__ xe, ElemMat<T, Traits<DIM>::NDE> K0,
                                const uint8_t* __restrict__ bcmask, T bcdiag, T* __restrict__ diag,
                                const T* __restrict__ cdiag) {
  constexpr int NDE = Traits<DIM>::NDE;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.nnodes()) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  T acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = T(0);
#pragma unroll
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int ei = i - 1 + ox, ej = j - 1 + oy, ek = (DIM == 3) ? k - 1 + oz : 0;
        if (ei < 0 || ei >= g.nx || ej < 0 || ej >= g.ny || ek < 0 || ek >= g.ez()) continue;
        const T x = xe[elem_id(g, ei, ej, ek)];
        const int ln = (1 - ox) + 2 * (1 - oy) + 4 * (DIM == 3 ? (1 - oz) : 0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = fma(x, K0.v[(ln * DIM + d) * NDE + ln * DIM + d], acc[d]);
      }
  const uint8_t m = bcmask ? bcmask[n] : 0;
#pragma unroll
  for (int d = 0; d < DIM; ++d)
    diag[n * DIM + d] = (((m >> d) & 1) ? bcdiag : acc[d]) + (cdiag ? cdiag[n * DIM + d] : T(0));
}

// ------------------------------------------------------------------------------------------ stencils
// Coefficient (d, c) of the block of node n at offset o, whose neighbour m = n + off(o) is clamped into the
// grid (`in`: the neighbour exists).  Forward offsets are stored at n, and their entries are exactly zero
// where the neighbour does not exist; a backward block is the transpose of the neighbour's stored forward
// block, read at the clamped index and replaced by zero when the neighbour does not exist, so that every
// load is unconditional and all of them can be in flight together.
// The DIM coefficients (d, 0..DIM-1) of row d of that block: base pointer and stride between them.
template <typename T>
struct StencilRow {
  const T* p;
  int stride;
};

template <typename T, int DIM>
__device__ __forceinline__ StencilRow<T> stencil_row(const T* __restrict__ S, int nn, int o, int d, int n, int m) {
  constexpr int CENTER = Traits<DIM>::CENTER, NOFF = Traits<DIM>::NOFF;
  if (o >= CENTER) return {S + (int64_t)(((o - CENTER) * DIM + d) * DIM) * nn + n, nn};
  return {S + (int64_t)((NOFF - 1 - o - CENTER) * DIM * DIM + d) * nn + m, DIM * nn};
}

template <typename T, int DIM>
__device__ __forceinline__ T stencil_coef(const T* __restrict__ S, int nn, int o, int d, int c, int n, int m, bool in) {
  const StencilRow<T> r = stencil_row<T, DIM>(S, nn, o, d, n, m);
  const T v = r.p[(int64_t)c * r.stride];
  return (o >= Traits<DIM>::CENTER || in) ? v : T(0);
}

// One thread per (component d, node n), d slowest so that the stencil loads of a warp are coalesced: the FP64
// products.  The bound of 4 CTAs per SM caps the registers at 64: enough to keep most of a row's 162 loads in
// flight (without it the compiler settles at 32 registers and each load is waited for; with 2 CTAs per SM the
// FP64 level-0 product loses occupancy: 265 vs 225 us).
template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(256, 4) stencil_apply_kernel(Grid g, const T* __restrict__ S, const T* __restrict__ u,
                                                            const T* __restrict__ b, const T* __restrict__ diag, T w,
                                                            T* __restrict__ y, ChebArgs<T> ch) {
  constexpr int NOFF = Traits<DIM>::NOFF;
  const int nn = (int)g.nnodes();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn * DIM) return;
  const int d = t / nn, n = t - d * nn;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  T acc = T(0);
#pragma unroll
  for (int o = 0; o < NOFF; ++o) {
    int dx, dy, dz;
    stencil_offset<DIM>(o, dx, dy, dz);
    const bool in = i + dx >= 0 && i + dx <= g.nx && j + dy >= 0 && j + dy <= g.ny && k + dz >= 0 && k + dz <= g.nz;
    const int ii = min(max(i + dx, 0), g.nx), jj = min(max(j + dy, 0), g.ny), kk = min(max(k + dz, 0), g.nz);
    const int m = (kk * (g.ny + 1) + jj) * (g.nx + 1) + ii;
    const StencilRow<T> row = stencil_row<T, DIM>(S, nn, o, d, n, m);
    const T* um = u + (int64_t)m * DIM;
    const bool live = o >= Traits<DIM>::CENTER || in;   // coefficient selects, not extra FP64 adds
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const T a = row.p[(int64_t)c * row.stride];
      acc = fma(live ? a : T(0), um[c], acc);
    }
  }
  const int64_t q = (int64_t)n * DIM + d;
  if (MODE == 0) {
    y[q] = acc;
  } else if (MODE == 1) {
    y[q] = b[q] - acc;
  } else if (MODE == 2) {
    y[q] = u[q] + w * ((b[q] - acc) / diag[q]);
  } else {
    const T a = (T)ch.coef[2 * ch.step], c = (T)ch.coef[2 * ch.step + 1];
    const T dn = (ch.step == 0 ? T(0) : a * ch.d[q]) + c * ((b[q] - acc) / diag[q]);
    ch.d[q] = dn;
    y[q] = u[q] + dn;
  }
}

// One thread per node: the DIM rows of the node together, so that each neighbour's DIM values are loaded once
// (a third of the value loads and of the index arithmetic of one thread per row).  Every row is summed in the
// same order as by stencil_apply_kernel (offsets, then components): the results are identical.
template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(256, 3) stencil_apply_node_kernel(Grid g, const T* __restrict__ S,
                                                                 const T* __restrict__ u, const T* __restrict__ b,
                                                                 const T* __restrict__ diag, T w, T* __restrict__ y,
                                                                 ChebArgs<T> ch) {
  constexpr int NOFF = Traits<DIM>::NOFF;
  const int nn = (int)g.nnodes();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  T acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = T(0);
#pragma unroll
  for (int o = 0; o < NOFF; ++o) {
    int dx, dy, dz;
    stencil_offset<DIM>(o, dx, dy, dz);
    const bool in = i + dx >= 0 && i + dx <= g.nx && j + dy >= 0 && j + dy <= g.ny && k + dz >= 0 && k + dz <= g.nz;
    const int ii = min(max(i + dx, 0), g.nx), jj = min(max(j + dy, 0), g.ny), kk = min(max(k + dz, 0), g.nz);
    const int m = (kk * (g.ny + 1) + jj) * (g.nx + 1) + ii;
    const bool live = o >= Traits<DIM>::CENTER || in;
    T um[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) um[c] = u[(int64_t)m * DIM + c];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const StencilRow<T> row = stencil_row<T, DIM>(S, nn, o, d, n, m);
#pragma unroll
      for (int c = 0; c < DIM; ++c) {
        const T a = row.p[(int64_t)c * row.stride];
        acc[d] = fma(live ? a : T(0), um[c], acc[d]);
      }
    }
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const int64_t q = (int64_t)n * DIM + d;
    if (MODE == 0) {
      y[q] = acc[d];
    } else if (MODE == 1) {
      y[q] = b[q] - acc[d];
    } else if (MODE == 2) {
      y[q] = u[q] + w * ((b[q] - acc[d]) / diag[q]);
    } else {
      const T a = (T)ch.coef[2 * ch.step], c = (T)ch.coef[2 * ch.step + 1];
      const T dn = (ch.step == 0 ? T(0) : a * ch.d[q]) + c * ((b[q] - acc[d]) / diag[q]);
      ch.d[q] = dn;
      y[q] = u[q] + dn;
    }
  }
}

// The same products for small levels, where one thread per row leaves most SMs idle and each thread waits
// through a long chain of dependent loads: the 3^dim offsets of a row are split over NOFF/3 threads (one
// x-line of 3 offsets each, so every thread issues its 3 DIM coefficient and 3 DIM value loads at once), and
// the partial sums are added in a fixed order in shared memory.  Block: 32 rows x NOFF/3 parts x SPLIT_G.
template <int DIM, int LINES>
struct SplitShape {
  static constexpr int P = Traits<DIM>::NOFF / 3 / LINES;   // parts per row (LINES x-lines each): 9 or 3 in 3D
  static constexpr int G = 288 / (32 * P);                  // 32-row groups per block
  static constexpr int THREADS = 32 * P * G;                // 288
};

template <typename T, int DIM, int MODE, int LINES>
__global__ void __launch_bounds__(SplitShape<DIM, LINES>::THREADS)
    stencil_apply_split_kernel(Grid g, const T* __restrict__ S, const T* __restrict__ u, const T* __restrict__ b,
                               const T* __restrict__ diag, T w, T* __restrict__ y, ChebArgs<T> ch) {
  constexpr int P = SplitShape<DIM, LINES>::P, G = SplitShape<DIM, LINES>::G;
  __shared__ T part[G][P][32];
  const int nn = (int)g.nnodes();
  const int lane = threadIdx.x, p = threadIdx.y, grp = threadIdx.z;
  const int t = (blockIdx.x * G + grp) * 32 + lane;
  const bool active = t < nn * DIM;
  const int d = active ? t / nn : 0, n = active ? t - d * nn : 0;
  const int64_t q = (int64_t)n * DIM + d;
  T bq = T(0), dq = T(1), uq = T(0), cq = T(0);
  if (active && p == 0) {   // epilogue operands, in flight together with the products
    if (MODE >= 1) bq = b[q];
    if (MODE >= 2) {
      dq = diag[q];
      uq = u[q];
    }
    if (MODE == 3 && ch.step != 0) cq = ch.d[q];
  }
  T acc = T(0);
  if (active) {
    int i, j, k;
    node_ijk(g, n, i, j, k);
#pragma unroll
    for (int li = 0; li < LINES; ++li) {
      const int l = p * LINES + li;     // x-line (dy, dz); the same across a warp: uniform branches
      const int dy = l % 3 - 1, dz = DIM == 3 ? l / 3 - 1 : 0;
      const bool in_yz = j + dy >= 0 && j + dy <= g.ny && k + dz >= 0 && k + dz <= g.nz;
      const int jj = min(max(j + dy, 0), g.ny), kk = min(max(k + dz, 0), g.nz);
      const int row = (kk * (g.ny + 1) + jj) * (g.nx + 1);
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int o = 3 * l + dx + 1;
        const bool in = in_yz && i + dx >= 0 && i + dx <= g.nx;
        const int m = row + min(max(i + dx, 0), g.nx);
        const StencilRow<T> srow = stencil_row<T, DIM>(S, nn, o, d, n, m);
        const T* um = u + (int64_t)m * DIM;
        const bool live = o >= Traits<DIM>::CENTER || in;
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          const T a = srow.p[(int64_t)c * srow.stride];
          acc = fma(live ? a : T(0), um[c], acc);
        }
      }
    }
  }
  part[grp][p][lane] = acc;
  __syncthreads();
  if (!active || p != 0) return;
  acc = T(0);
#pragma unroll
  for (int r = 0; r < P; ++r) acc += part[grp][r][lane];
  if (MODE == 0) {
    y[q] = acc;
  } else if (MODE == 1) {
    y[q] = bq - acc;
  } else if (MODE == 2) {
    y[q] = uq + w * ((bq - acc) / dq);
  } else {
    const T a = (T)ch.coef[2 * ch.step], c = (T)ch.coef[2 * ch.step + 1];
    const T dn = a * cq + c * ((bq - acc) / dq);
    ch.d[q] = dn;
    y[q] = uq + dn;
  }
}

template <typename T, int DIM>
__global__ void stencil_diag_kernel(Grid g, const T* __restrict__ S, T* __restrict__ diag) {
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
#pragma unroll
  for (int d = 0; d < DIM; ++d) diag[n * DIM + d] = S[((int64_t)d * DIM + d) * nn + n];   // centre block, h = 0
}

// centre block diagonal of the stencils += c (a constant diagonal added to the operator)
template <typename T, int DIM>
__global__ void stencil_add_diag_kernel(Grid g, T* __restrict__ S, const T* __restrict__ c) {
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
#pragma unroll
  for (int d = 0; d < DIM; ++d) S[((int64_t)d * DIM + d) * nn + n] += c[n * DIM + d];
}

// Row sums of |A| of a stencil operator, per dof (the l1-Jacobi diagonal: with it the spectrum of
// D_l1^-1 A lies in (0, 1] by Gershgorin's theorem, whatever the contrast of the element scaling).
template <typename T, int DIM>
__global__ void __launch_bounds__(256) stencil_rowabs_kernel(Grid g, const T* __restrict__ S, T* __restrict__ out) {
  constexpr int NOFF = Traits<DIM>::NOFF;
  const int nn = (int)g.nnodes();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn * DIM) return;
  const int d = t / nn, n = t - d * nn;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  T sum = T(0);
#pragma unroll
  for (int o = 0; o < NOFF; ++o) {
    int dx, dy, dz;
    stencil_offset<DIM>(o, dx, dy, dz);
    const bool in = i + dx >= 0 && i + dx <= g.nx && j + dy >= 0 && j + dy <= g.ny && k + dz >= 0 && k + dz <= g.nz;
    const int m = (min(max(k + dz, 0), g.nz) * (g.ny + 1) + min(max(j + dy, 0), g.ny)) * (g.nx + 1) +
                  min(max(i + dx, 0), g.nx);
#pragma unroll
    for (int c = 0; c < DIM; ++c) sum += fabs(stencil_coef<T, DIM>(S, nn, o, d, c, n, m, in));
  }
  out[(int64_t)n * DIM + d] = sum;
}

// ------------------------------------------------------------------------------------------ transfers
// weight of a fine node at signed offset a (in fine units) from a coarse node: 1 at 0, 1/2 at +-1
__device__ __forceinline__ double tw(int a) { return a == 0 ? 1.0 : 0.5; }

// rc = R^T rf: one thread per coarse node N (all DIM components: one set of index arithmetic, contiguous
// component loads), gathering the 3^dim fine neighbours of the coarse node with branch-free clamped loads
// (weight zero outside the grid).
template <typename T, int DIM>
__global__ void __launch_bounds__(256) restrict_kernel(Grid gf, const T* __restrict__ rf, T* __restrict__ rc) {
  const Grid gc = gf.coarse();
  const int ncn = (int)gc.nnodes();
  const int N = blockIdx.x * blockDim.x + threadIdx.x;
  if (N >= ncn) return;
  int I, J, K;
  node_ijk(gc, N, I, J, K);
  T acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = T(0);
#pragma unroll
  for (int c = (DIM == 3 ? -1 : 0); c <= (DIM == 3 ? 1 : 0); ++c)
#pragma unroll
    for (int bb = -1; bb <= 1; ++bb)
#pragma unroll
      for (int a = -1; a <= 1; ++a) {
        const int i = 2 * I + a, j = 2 * J + bb, k = 2 * K + c;
        const bool in = i >= 0 && i <= gf.nx && j >= 0 && j <= gf.ny && k >= 0 && k <= gf.nz;
        const T wgt = in ? (T)(tw(a) * tw(bb) * tw(c)) : T(0);
        const int m = (min(max(k, 0), gf.nz) * (gf.ny + 1) + min(max(j, 0), gf.ny)) * (gf.nx + 1) + min(max(i, 0), gf.nx);
        const T* src = rf + (int64_t)m * DIM;
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = fma(wgt, src[d], acc[d]);
      }
#pragma unroll
  for (int d = 0; d < DIM; ++d) rc[(int64_t)N * DIM + d] = acc[d];
}

// uf += R uc: one thread per fine node n (all DIM components); the 2^dim candidate parents are read at
// clamped indices with weight zero where a parent does not exist (even coordinate).
template <typename T, int DIM>
__global__ void __launch_bounds__(256) prolong_add_kernel(Grid gf, const T* __restrict__ uc, T* __restrict__ uf) {
  const Grid gc = gf.coarse();
  const int nfn = (int)gf.nnodes();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nfn) return;
  int i, j, k;
  node_ijk(gf, n, i, j, k);
  const int i0 = i >> 1, j0 = j >> 1, k0 = k >> 1;
  const int i1 = i0 + (i & 1), j1 = j0 + (j & 1), k1 = k0 + (k & 1);
  const T wx0 = (i & 1) ? T(0.5) : T(1), wx1 = (i & 1) ? T(0.5) : T(0);
  const T wy0 = (j & 1) ? T(0.5) : T(1), wy1 = (j & 1) ? T(0.5) : T(0);
  const T wz0 = (DIM == 3 && (k & 1)) ? T(0.5) : T(1), wz1 = (DIM == 3 && (k & 1)) ? T(0.5) : T(0);
  const int cx = gc.nx + 1, cxy = (gc.nx + 1) * (gc.ny + 1);
  const int par[8] = {k0 * cxy + j0 * cx + i0, k0 * cxy + j0 * cx + i1, k0 * cxy + j1 * cx + i0,
                      k0 * cxy + j1 * cx + i1, k1 * cxy + j0 * cx + i0, k1 * cxy + j0 * cx + i1,
                      k1 * cxy + j1 * cx + i0, k1 * cxy + j1 * cx + i1};
  const T wgt[8] = {wz0 * wy0 * wx0, wz0 * wy0 * wx1, wz0 * wy1 * wx0, wz0 * wy1 * wx1,
                    wz1 * wy0 * wx0, wz1 * wy0 * wx1, wz1 * wy1 * wx0, wz1 * wy1 * wx1};
  T* dst = uf + (int64_t)n * DIM;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    T acc = T(0);
#pragma unroll
    for (int p = 0; p < (DIM == 3 ? 8 : 4); ++p) acc = fma(wgt[p], uc[(int64_t)par[p] * DIM + d], acc);
    dst[d] += acc;
  }
}

// ------------------------------------------------------------------------------------------ Galerkin
// 1D interpolation from the 2 coarse nodes A of a coarse cell to the fine local node a of child s:
// fine position (s + a) / 2 in coarse-cell units.
__host__ __device__ __forceinline__ double p1(int s, int a, int A) {
  const int pos2 = s + a;  // 0, 1, 2  -> position 0, 1/2, 1
  if (pos2 == 1) return 0.5;
  return (pos2 == 0) == (A == 0) ? 1.0 : 0.0;
}

// E(NDE x NDE, smem) += M_s^T K M_s where M_s maps coarse-cell dofs to the dofs of child s.
// Sum factorisation: transform row index then column index, one axis at a time.  buf/buf2: NDE*NDE.
template <typename T, int DIM>
__device__ void galerkin_child_accumulate(T* E, T* K, T* buf, int s) {
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  // For a dof index q = node*DIM + d with node = ax + 2 ay + 4 az, transforming axis `ax_id` replaces the
  // bit of that axis (fine local) by the coarse bit: out[..A..] = sum_a p1(s_ax, a, A) in[..a..].
  T* src = K;
  T* dst = buf;
#pragma unroll 1
  for (int side = 0; side < 2; ++side) {
#pragma unroll 1
    for (int axis = 0; axis < DIM; ++axis) {
      const int sa = (s >> axis) & 1;
      for (int e = threadIdx.x; e < NE; e += blockDim.x) {
        const int r = e / NDE, c = e % NDE;
        const int q = side == 0 ? r : c;
        const int node = q / DIM, d = q % DIM;
        const int A = (node >> axis) & 1;
        T v = T(0);
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          const double wgt = p1(sa, a, A);
          if (wgt != 0.0) {
            const int qa = ((node & ~(1 << axis)) | (a << axis)) * DIM + d;
            const int idx = side == 0 ? qa * NDE + c : r * NDE + qa;
            v = fma((T)wgt, src[idx], v);
          }
        }
        dst[e] = v;
      }
      __syncthreads();
      T* t = src;
      src = dst;
      dst = t;
    }
  }
  // after 2*DIM passes (even) the result is back in K
  for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] += src[e];
  __syncthreads();
}

// Level-1 coarse element matrices from the matrix-free fine operator.
// Persistent CTAs of 8 warps walk the coarse elements 8 at a time, one warp per coarse element: if no node
// of its children is constrained (the common case) the warp writes E = sum_c x_c (M_c^T K0 M_c) from the
// precomputed table (staged in shared memory), 18 entries per lane in 3D.  Coarse elements touching a
// Dirichlet dof are queued and then transformed by the whole CTA: unconstrained children from the table,
// the others with their masked matrix plus the bcdiag terms of the fine Dirichlet dofs assigned to them
// (each fine node is assigned to the element min(i, nx-1), ...), by sum factorisation.
constexpr int GAL_THREADS = 256;
constexpr int GAL_WARPS = GAL_THREADS / 32;

template <typename T, int DIM>
__global__ void __launch_bounds__(GAL_THREADS) galerkin_from_ebe_kernel(Grid gf, const T* __restrict__ xe,
                                                                        ElemMat<T, Traits<DIM>::NDE> K0,
                                                                        const uint8_t* __restrict__ bcmask, T bcdiag,
                                                                        const T* __restrict__ table,
                                                                        T* __restrict__ Ec, unsigned perm,
                                                                        int listed) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  constexpr int PER_LANE = (NE + 31) / 32;
  extern __shared__ __align__(16) unsigned char gal_smem[];
  T* tab = reinterpret_cast<T*>(gal_smem);   // [NN][NE]
  T* E = tab + NN * NE;
  T* Kc = E + NE;
  T* buf = Kc + NE;
  T* K0s = buf + NE;                         // K0 in shared memory: the slow path reads it at per-thread indices
  __shared__ T xs[NN];
  __shared__ uint8_t cmask[NN][NN];
  __shared__ int queue[GAL_WARPS];
  __shared__ int nqueue;
  const Grid gc = gf.coarse();
  const int nelc = (int)gc.nel();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < NN * NE; e += blockDim.x) tab[e] = table[e];
  for (int e = threadIdx.x; e < NE; e += blockDim.x) K0s[e] = K0.v[e];
  if (threadIdx.x == 0) nqueue = 0;
  __syncthreads();
  for (int base = blockIdx.x * GAL_WARPS; base < nelc; base += gridDim.x * GAL_WARPS) {
    // elements visited in a permuted order (perm coprime to the count): constrained elements, which take
    // the slow path, spread over all CTAs instead of following the period of the grid
    const int lin = base + warp;
    const int ec = lin < nelc ? (int)(((uint64_t)lin * perm) % (uint64_t)nelc) : nelc;
    if (lin < nelc) {
      const int CI = ec % gc.nx, CJ = (ec / gc.nx) % gc.ny, CK = ec / (gc.nx * gc.ny);
      // children's x (lanes 0..NN-1) and any constrained node of the children (NN*NN pairs over the lanes)
      T xv = T(0);
      if (lane < NN)
        xv = xe[elem_id(gf, 2 * CI + (lane & 1), 2 * CJ + ((lane >> 1) & 1), DIM == 3 ? 2 * CK + ((lane >> 2) & 1) : 0)];
      int mine = 0;
      for (int q = lane; q < NN * NN; q += 32) {
        const int sc = q / NN, a = q % NN;
        const int ni = 2 * CI + (sc & 1) + (a & 1), nj = 2 * CJ + ((sc >> 1) & 1) + ((a >> 1) & 1);
        const int nk = DIM == 3 ? 2 * CK + ((sc >> 2) & 1) + ((a >> 2) & 1) : 0;
        mine |= (bcmask ? bcmask[node_id(gf, ni, nj, nk)] : 0) != 0;
      }
      if (__any_sync(0xffffffffu, mine)) {
        // constrained element: left to galerkin_listed_kernel when the caller lists them, else queued here
        if (lane == 0 && !listed) queue[atomicAdd(&nqueue, 1)] = ec;
      } else {
        T xc[NN];
#pragma unroll
        for (int sc = 0; sc < NN; ++sc) xc[sc] = __shfl_sync(0xffffffffu, xv, sc);
        T* out = Ec + (int64_t)ec * NE;
#pragma unroll
        for (int k = 0; k < PER_LANE; ++k) {
          const int e = lane + 32 * k;
          if (e < NE) {
            T v = T(0);
#pragma unroll
            for (int sc = 0; sc < NN; ++sc) v = fma(xc[sc], tab[sc * NE + e], v);
            out[e] = v;
          }
        }
      }
    }
    __syncthreads();
    const int nq = nqueue;
    for (int qi = 0; qi < nq; ++qi) {
      const int ecq = queue[qi];
      const int CI = ecq % gc.nx, CJ = (ecq / gc.nx) % gc.ny, CK = ecq / (gc.nx * gc.ny);
      for (int q = threadIdx.x; q < NN * NN; q += blockDim.x) {
        const int sc = q / NN, a = q % NN;
        const int ni = 2 * CI + (sc & 1) + (a & 1), nj = 2 * CJ + ((sc >> 1) & 1) + ((a >> 1) & 1);
        const int nk = DIM == 3 ? 2 * CK + ((sc >> 2) & 1) + ((a >> 2) & 1) : 0;
        cmask[sc][a] = bcmask ? bcmask[node_id(gf, ni, nj, nk)] : 0;
      }
      if (threadIdx.x < NN) {
        const int sc = threadIdx.x;
        xs[sc] = xe[elem_id(gf, 2 * CI + (sc & 1), 2 * CJ + ((sc >> 1) & 1), DIM == 3 ? 2 * CK + ((sc >> 2) & 1) : 0)];
      }
      for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] = T(0);
      __syncthreads();
      for (int sidx = 0; sidx < NN; ++sidx) {
        const int fi = 2 * CI + (sidx & 1), fj = 2 * CJ + ((sidx >> 1) & 1), fk = DIM == 3 ? 2 * CK + ((sidx >> 2) & 1) : 0;
        const T x = xs[sidx];
        bool child_bc = false;
#pragma unroll
        for (int a = 0; a < NN; ++a) child_bc |= cmask[sidx][a] != 0;
        if (!child_bc) {
          for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] = fma(x, tab[sidx * NE + e], E[e]);
          __syncthreads();
          continue;
        }
        for (int e = threadIdx.x; e < NE; e += blockDim.x) {
          const int r = e / NDE, c = e % NDE;
          const int rn = r / DIM, rd = r % DIM, cn = c / DIM, cd = c % DIM;
          const bool rb = (cmask[sidx][rn] >> rd) & 1, cb = (cmask[sidx][cn] >> cd) & 1;
          T v = (rb || cb) ? T(0) : x * K0s[e];
          if (r == c && rb) {
            const int ni = fi + (rn & 1), nj = fj + ((rn >> 1) & 1), nk = DIM == 3 ? fk + ((rn >> 2) & 1) : 0;
            const int ai = min(ni, gf.nx - 1), aj = min(nj, gf.ny - 1), ak = DIM == 3 ? min(nk, gf.nz - 1) : 0;
            if (ai == fi && aj == fj && ak == fk) v = bcdiag;
          }
          Kc[e] = v;
        }
        __syncthreads();
        galerkin_child_accumulate<T, DIM>(E, Kc, buf, sidx);
      }
      for (int e = threadIdx.x; e < NE; e += blockDim.x) Ec[(int64_t)ecq * NE + e] = E[e];
      __syncthreads();
    }
    if (threadIdx.x == 0) nqueue = 0;
    __syncthreads();
  }
}

// The coarse elements with a constrained node, listed by the caller (fixed for a problem): one CTA each,
// spread over the whole GPU.  Unconstrained children from the table, constrained ones by their masked
// matrix plus bcdiag on the fine Dirichlet dofs assigned to them, transformed by sum factorisation.
template <typename T, int DIM>
__global__ void __launch_bounds__(GAL_THREADS) galerkin_listed_kernel(Grid gf, const T* __restrict__ xe,
                                                                      ElemMat<T, Traits<DIM>::NDE> K0,
                                                                      const uint8_t* __restrict__ bcmask, T bcdiag,
                                                                      const T* __restrict__ table,
                                                                      const int32_t* __restrict__ list,
                                                                      T* __restrict__ Ec) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  extern __shared__ __align__(16) unsigned char gal_smem[];
  T* E = reinterpret_cast<T*>(gal_smem);
  T* Kc = E + NE;
  T* buf = Kc + NE;
  T* K0s = buf + NE;
  __shared__ T xs[NN];
  __shared__ uint8_t cmask[NN][NN];
  const Grid gc = gf.coarse();
  const int ecq = list[blockIdx.x];
  const int CI = ecq % gc.nx, CJ = (ecq / gc.nx) % gc.ny, CK = ecq / (gc.nx * gc.ny);
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    K0s[e] = K0.v[e];
    E[e] = T(0);
  }
  for (int q = threadIdx.x; q < NN * NN; q += blockDim.x) {
    const int sc = q / NN, a = q % NN;
    const int ni = 2 * CI + (sc & 1) + (a & 1), nj = 2 * CJ + ((sc >> 1) & 1) + ((a >> 1) & 1);
    const int nk = DIM == 3 ? 2 * CK + ((sc >> 2) & 1) + ((a >> 2) & 1) : 0;
    cmask[sc][a] = bcmask ? bcmask[node_id(gf, ni, nj, nk)] : 0;
  }
  if (threadIdx.x < NN) {
    const int sc = threadIdx.x;
    xs[sc] = xe[elem_id(gf, 2 * CI + (sc & 1), 2 * CJ + ((sc >> 1) & 1), DIM == 3 ? 2 * CK + ((sc >> 2) & 1) : 0)];
  }
  __syncthreads();
  for (int sidx = 0; sidx < NN; ++sidx) {
    const int fi = 2 * CI + (sidx & 1), fj = 2 * CJ + ((sidx >> 1) & 1), fk = DIM == 3 ? 2 * CK + ((sidx >> 2) & 1) : 0;
    const T x = xs[sidx];
    bool child_bc = false;
#pragma unroll
    for (int a = 0; a < NN; ++a) child_bc |= cmask[sidx][a] != 0;
    if (!child_bc) {
      for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] = fma(x, table[sidx * NE + e], E[e]);
      __syncthreads();
      continue;
    }
    for (int e = threadIdx.x; e < NE; e += blockDim.x) {
      const int r = e / NDE, c = e % NDE;
      const int rn = r / DIM, rd = r % DIM, cn = c / DIM, cd = c % DIM;
      const bool rb = (cmask[sidx][rn] >> rd) & 1, cb = (cmask[sidx][cn] >> cd) & 1;
      T v = (rb || cb) ? T(0) : x * K0s[e];
      if (r == c && rb) {
        const int ni = fi + (rn & 1), nj = fj + ((rn >> 1) & 1), nk = DIM == 3 ? fk + ((rn >> 2) & 1) : 0;
        const int ai = min(ni, gf.nx - 1), aj = min(nj, gf.ny - 1), ak = DIM == 3 ? min(nk, gf.nz - 1) : 0;
        if (ai == fi && aj == fj && ak == fk) v = bcdiag;
      }
      Kc[e] = v;
    }
    __syncthreads();
    galerkin_child_accumulate<T, DIM>(E, Kc, buf, sidx);
  }
  for (int e = threadIdx.x; e < NE; e += blockDim.x) Ec[(int64_t)ecq * NE + e] = E[e];
}

// Next-level coarse element matrices from element matrices Ef of grid gf: E_C = sum_c M_c^T E_c M_c, where
// M_c maps the coarse element's dofs to those of child c (trilinear weights).  One warp per coarse element,
// children one after the other, no CTA barriers: lane a forms row a of T = E_c M_c (one column J at a time,
// so the trip count over the nonzeros of column J of M_c is uniform across the warp), then lane J adds
// column J of M_c^T T (one row I at a time) to its column of E_C, kept in registers.  The nonzeros of M_c
// (child c, coarse node N -> fine nodes with nonzero weight) come from a table in shared memory.
template <typename T, int DIM>
__global__ void __launch_bounds__(GAL_THREADS) galerkin_from_elements_kernel(Grid gf, const T* __restrict__ Ef,
                                                                             T* __restrict__ Ec) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  constexpr int PITCH = NDE + 1;   // odd row pitch: lanes reading one column hit distinct banks
  extern __shared__ __align__(16) unsigned char g_smem[];
  __shared__ int8_t sup_cnt[NN][NN];
  __shared__ int8_t sup_node[NN][NN][NN];
  __shared__ T sup_w[NN][NN][NN];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* Es = reinterpret_cast<T*>(g_smem) + (size_t)warp * (NDE * PITCH + NE);   // child matrix, padded rows
  T* Ts = Es + NDE * PITCH;                                                     // T = E_c M_c, [a][J]
  if (threadIdx.x < NN * NN) {
    const int c = threadIdx.x / NN, N = threadIdx.x % NN;
    int cnt = 0;
    for (int a = 0; a < NN; ++a) {
      double w = 1.0;
#pragma unroll
      for (int ax = 0; ax < DIM; ++ax) w *= p1((c >> ax) & 1, (a >> ax) & 1, (N >> ax) & 1);
      if (w != 0.0) {
        sup_node[c][N][cnt] = (int8_t)a;
        sup_w[c][N][cnt] = (T)w;
        ++cnt;
      }
    }
    sup_cnt[c][N] = (int8_t)cnt;
  }
  __syncthreads();
  const Grid gc = gf.coarse();
  const int nelc = (int)gc.nel();
  const int nwarps = gridDim.x * GAL_WARPS;
  for (int ec = blockIdx.x * GAL_WARPS + warp; ec < nelc; ec += nwarps) {
    const int CI = ec % gc.nx, CJ = (ec / gc.nx) % gc.ny, CK = ec / (gc.nx * gc.ny);
    T acc[NDE];
#pragma unroll
    for (int I = 0; I < NDE; ++I) acc[I] = T(0);
    for (int c = 0; c < NN; ++c) {
      const int64_t child = elem_id(gf, 2 * CI + (c & 1), 2 * CJ + ((c >> 1) & 1), DIM == 3 ? 2 * CK + ((c >> 2) & 1) : 0);
      const T* src = Ef + child * NE;
      for (int e = lane; e < NE; e += 32) {
        const int r = e / NDE;
        Es[r * PITCH + (e - r * NDE)] = src[e];
      }
      __syncwarp();
      if (lane < NDE) {
#pragma unroll 1
        for (int J = 0; J < NDE; ++J) {
          const int NJ = J / DIM, dJ = J - NJ * DIM;
          const int cnt = sup_cnt[c][NJ];
          T v = T(0);
          for (int k = 0; k < cnt; ++k) v = fma(sup_w[c][NJ][k], Es[lane * PITCH + sup_node[c][NJ][k] * DIM + dJ], v);
          Ts[lane * NDE + J] = v;
        }
      }
      __syncwarp();
      if (lane < NDE) {
#pragma unroll
        for (int I = 0; I < NDE; ++I) {
          const int NI = I / DIM, dI = I - NI * DIM;
          const int cnt = sup_cnt[c][NI];
          T v = acc[I];
          for (int k = 0; k < cnt; ++k) v = fma(sup_w[c][NI][k], Ts[(sup_node[c][NI][k] * DIM + dI) * NDE + lane], v);
          acc[I] = v;
        }
      }
      __syncwarp();
    }
    if (lane < NDE) {
      T* out = Ec + (int64_t)ec * NE;
#pragma unroll
      for (int I = 0; I < NDE; ++I) out[I * NDE + lane] = acc[I];
    }
  }
}

// Node stencils from element matrices: thread per (node n = x index, stored offset h = blockIdx.y).
template <typename T, int DIM>
__global__ void stencil_from_elements_kernel(Grid g, const T* __restrict__ E, T* __restrict__ S) {
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int h = blockIdx.y, o = Traits<DIM>::CENTER + h;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  int dx, dy, dz;
  stencil_offset<DIM>(o, dx, dy, dz);
  T acc[DIM * DIM];
#pragma unroll
  for (int q = 0; q < DIM * DIM; ++q) acc[q] = T(0);
#pragma unroll
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int ei = i - 1 + ox, ej = j - 1 + oy, ek = DIM == 3 ? k - 1 + oz : 0;
        if (ei < 0 || ei >= g.nx || ej < 0 || ej >= g.ny || ek < 0 || ek >= g.ez()) continue;
        // local coordinates of n and m = n + (dx,dy,dz) in this element
        const int lx = 1 - ox, ly = 1 - oy, lz = DIM == 3 ? 1 - oz : 0;
        const int mx = lx + dx, my = ly + dy, mz = lz + dz;
        if (mx < 0 || mx > 1 || my < 0 || my > 1 || mz < 0 || mz > 1) continue;
        const int ln = lx + 2 * ly + 4 * lz, lm = mx + 2 * my + 4 * mz;
        const T* Ee = E + elem_id(g, ei, ej, ek) * NE;
#pragma unroll
        for (int d = 0; d < DIM; ++d)
#pragma unroll
          for (int c = 0; c < DIM; ++c) acc[d * DIM + c] += Ee[(ln * DIM + d) * NDE + lm * DIM + c];
      }
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int c = 0; c < DIM; ++c) S[((int64_t)(h * DIM + d) * DIM + c) * nn + n] = acc[d * DIM + c];
}

// Level-0 node stencils of K(x) (Dirichlet rows: bcdiag on the diagonal only; Dirichlet columns: zero).
// Thread per (offset o, node n): sums x_e K0[ln, lm] over the elements containing n and m = n + o.
template <typename T, int DIM>
__global__ void ebe_stencil_kernel(Grid g, const T* __restrict__ xe, ElemMat<T, Traits<DIM>::NDE> K0,
                                   const uint8_t* __restrict__ bcmask, T bcdiag, T* __restrict__ S) {
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int CENTER = Traits<DIM>::CENTER;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int h = blockIdx.y, o = CENTER + h;   // stored (forward) offsets only: half the FP64 work
  int i, j, k;
  node_ijk(g, n, i, j, k);
  int dx, dy, dz;
  stencil_offset<DIM>(o, dx, dy, dz);
  const int ii = i + dx, jj = j + dy, kk = k + dz;
  const bool nbr_in = ii >= 0 && ii <= g.nx && jj >= 0 && jj <= g.ny && kk >= 0 && kk <= g.nz;
  const uint8_t mrow = bcmask ? bcmask[n] : 0;
  const uint8_t mcol = (bcmask && nbr_in) ? bcmask[node_id(g, ii, jj, kk)] : 0;
  T acc[DIM * DIM];
#pragma unroll
  for (int q = 0; q < DIM * DIM; ++q) acc[q] = T(0);
  if (nbr_in) {
#pragma unroll
    for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
      for (int oy = 0; oy < 2; ++oy)
#pragma unroll
        for (int ox = 0; ox < 2; ++ox) {
          const int ei = i - 1 + ox, ej = j - 1 + oy, ek = DIM == 3 ? k - 1 + oz : 0;
          if (ei < 0 || ei >= g.nx || ej < 0 || ej >= g.ny || ek < 0 || ek >= g.ez()) continue;
          const int lx = 1 - ox, ly = 1 - oy, lz = DIM == 3 ? 1 - oz : 0;
          const int mx = lx + dx, my = ly + dy, mz = lz + dz;
          if (mx < 0 || mx > 1 || my < 0 || my > 1 || mz < 0 || mz > 1) continue;
          const int ln = lx + 2 * ly + 4 * lz, lm = mx + 2 * my + 4 * mz;
          const T x = xe[elem_id(g, ei, ej, ek)];
#pragma unroll
          for (int d = 0; d < DIM; ++d)
#pragma unroll
            for (int c = 0; c < DIM; ++c) acc[d * DIM + c] = fma(x, K0.v[(ln * DIM + d) * NDE + lm * DIM + c], acc[d * DIM + c]);
        }
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      T v = acc[d * DIM + c];
      if (((mrow >> d) & 1) || ((mcol >> c) & 1)) v = T(0);
      if (((mrow >> d) & 1) && o == CENTER && c == d) v = bcdiag;
      S[((int64_t)(h * DIM + d) * DIM + c) * nn + n] = v;
    }
}

template <typename T, int DIM>
__global__ void stencil_to_dense_kernel(Grid g, const T* __restrict__ S, const int32_t* __restrict__ pos,
                                        double* __restrict__ A) {
  const int64_t nn = g.nnodes();
  const int64_t ndof = nn * DIM;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int h = blockIdx.y, o = Traits<DIM>::CENTER + h;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  int dx, dy, dz;
  stencil_offset<DIM>(o, dx, dy, dz);
  const int ii = i + dx, jj = j + dy, kk = k + dz;
  if (ii < 0 || ii > g.nx || jj < 0 || jj > g.ny || kk < 0 || kk > g.nz) return;
  const int64_t m = node_id(g, ii, jj, kk);
  // the stored block (n, m) and, for a forward offset, its transpose (m, n): every entry written once
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const int64_t row = pos ? pos[n * DIM + d] : n * DIM + d, col = pos ? pos[m * DIM + c] : m * DIM + c;
      const double v = (double)S[((int64_t)(h * DIM + d) * DIM + c) * nn + n];
      A[row * ndof + col] = v;
      if (h > 0) A[col * ndof + row] = v;
    }
}

__global__ void dofconn_kernel(Grid g, int64_t* __restrict__ dc) {
  const int dim = g.dim();
  const int nn = 1 << dim;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.nel()) return;
  const int i = (int)(e % g.nx), j = (int)((e / g.nx) % g.ny), k = (int)(e / ((int64_t)g.nx * g.ny));
  for (int a = 0; a < nn; ++a) {
    const int64_t nd = node_id(g, i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1));
    for (int d = 0; d < dim; ++d) dc[e * nn * dim + a * dim + d] = nd * dim + d;
  }
}

// ------------------------------------------------------------------------------------------ dispatch
// Implementation of the FP32 3D operator (pmg_set_operator_kernel): CUDA-core FMAs by default.
static std::atomic<int> g_f32_operator{PMG_OPERATOR_FMA};

int ebe_apply_f32_3d(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                     const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                     const float* cdiag, cudaStream_t st) {
  const int kind = g_f32_operator.load(std::memory_order_relaxed);
  if (kind == PMG_OPERATOR_TCGEN05)
    return ebe_apply_tc_f32(mode, g, xe, K0, bcmask, bcdiag, u, b, diag, w, y, ch, cdiag, st);
  return ebe_apply_fma_f32(mode, g, xe, K0, bcmask, bcdiag, u, b, diag, w, y, ch, cdiag, st);
}

template <typename T, int DIM>
int ebe_apply_t(int mode, Grid g, const void* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                const void* u, const void* b, const void* diag, double w, void* y, const void* cdiag, cudaStream_t st) {
  if constexpr (DIM == 3 && sizeof(T) == 4)
    return ebe_apply_f32_3d(mode, g, (const float*)xe, K0, bcmask, bcdiag, (const float*)u, (const float*)b,
                            (const float*)diag, w, (float*)y, ChebArgs<float>{nullptr, nullptr, 0}, (const float*)cdiag,
                            st);
  const T* c_ = (const T*)cdiag;
  auto K = make_elem_mat<T, Traits<DIM>::NDE>(K0);
  if constexpr (DIM == 3) {
    const dim3 block(TBX, TBY, TBZ);
    const dim3 grid((g.nx + 1 + TBX - 1) / TBX, (g.ny + 1 + TBY - 1) / TBY, (g.nz + 1 + TBZ - 1) / TBZ);
    const T* xe_ = (const T*)xe;
    const T* u_ = (const T*)u;
    const T* b_ = (const T*)b;
    const T* d_ = (const T*)diag;
    T* y_ = (T*)y;
    if (mode == PMG_APPLY_MATVEC)
      ebe_apply_tiled_kernel<T, 0><<<grid, block, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_, c_);
    else if (mode == PMG_APPLY_RESIDUAL)
      ebe_apply_tiled_kernel<T, 1><<<grid, block, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_, c_);
    else
      ebe_apply_tiled_kernel<T, 2><<<grid, block, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_, c_);
    return check_launch();
  }
  const int threads = 128;
  const unsigned blocks = blocks_for(g.nnodes(), threads);
  const T* xe_ = (const T*)xe;
  const T* u_ = (const T*)u;
  const T* b_ = (const T*)b;
  const T* d_ = (const T*)diag;
  T* y_ = (T*)y;
  if (mode == PMG_APPLY_MATVEC)
    ebe_apply_kernel<T, DIM, 0><<<blocks, threads, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_, c_);
  else if (mode == PMG_APPLY_RESIDUAL)
    ebe_apply_kernel<T, DIM, 1><<<blocks, threads, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_, c_);
  else
    ebe_apply_kernel<T, DIM, 2><<<blocks, threads, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_, c_);
  return check_launch();
}

// Levels with at most this many rows use the split-row kernel with one x-line per part (9 parts per 3D row);
// larger levels one row per thread (measured at 64x32x32: 10.1 us per product against 12.4 us with one z-plane
// of 9 offsets per part and 15.5 us with one x-line per part).
constexpr int64_t SPLIT_MAX_ROWS = int64_t(1) << 16;

template <typename T, int DIM, int LINES>
int split_apply(int mode, Grid g, int64_t rows, const T* S, const T* u, const T* b, const T* d, T w, T* y,
                ChebArgs<T> ch, cudaStream_t st) {
  using SS = SplitShape<DIM, LINES>;
  const dim3 blk(32, SS::P, SS::G);
  const unsigned nb = blocks_for(rows, 32 * SS::G);
  if (mode == PMG_APPLY_MATVEC)
    stencil_apply_split_kernel<T, DIM, 0, LINES><<<nb, blk, 0, st>>>(g, S, u, b, d, w, y, ch);
  else if (mode == PMG_APPLY_RESIDUAL)
    stencil_apply_split_kernel<T, DIM, 1, LINES><<<nb, blk, 0, st>>>(g, S, u, b, d, w, y, ch);
  else if (mode == PMG_APPLY_JACOBI)
    stencil_apply_split_kernel<T, DIM, 2, LINES><<<nb, blk, 0, st>>>(g, S, u, b, d, w, y, ch);
  else
    stencil_apply_split_kernel<T, DIM, 3, LINES><<<nb, blk, 0, st>>>(g, S, u, b, d, w, y, ch);
  return check_launch();
}

template <typename T, int DIM>
int stencil_apply_t(int mode, Grid g, const void* S, const void* u, const void* b, const void* diag, double w,
                    void* y, cudaStream_t st, ChebArgs<T> ch = ChebArgs<T>{nullptr, nullptr, 0}) {
  const int threads = 256;
  const int64_t rows = g.nnodes() * DIM;
  const unsigned blocks = blocks_for(rows, threads);
  const T* S_ = (const T*)S;
  const T* u_ = (const T*)u;
  const T* b_ = (const T*)b;
  const T* d_ = (const T*)diag;
  T* y_ = (T*)y;
  if (rows <= SPLIT_MAX_ROWS) return split_apply<T, DIM, 1>(mode, g, rows, S_, u_, b_, d_, (T)w, y_, ch, st);
  if constexpr (std::is_same<T, double>::value) {
    // FP64 (the outer level-0 product): bound by the FP64 pipe, where a thread per row keeps more warps resident
    // (232 us against 236 us with a thread per node at 128 x 64 x 64)
    if (mode == PMG_APPLY_MATVEC)
      stencil_apply_kernel<T, DIM, 0><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    else if (mode == PMG_APPLY_RESIDUAL)
      stencil_apply_kernel<T, DIM, 1><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    else if (mode == PMG_APPLY_JACOBI)
      stencil_apply_kernel<T, DIM, 2><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    else
      stencil_apply_kernel<T, DIM, 3><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    return check_launch();
  } else {
    // FP32 (level 1 of the mixed hierarchy): a thread per node, 17.0 us against 21.1 us at 64 x 32 x 32
    const unsigned nblocks = blocks_for(g.nnodes(), threads);
    if (mode == PMG_APPLY_MATVEC)
      stencil_apply_node_kernel<T, DIM, 0><<<nblocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    else if (mode == PMG_APPLY_RESIDUAL)
      stencil_apply_node_kernel<T, DIM, 1><<<nblocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    else if (mode == PMG_APPLY_JACOBI)
      stencil_apply_node_kernel<T, DIM, 2><<<nblocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    else
      stencil_apply_node_kernel<T, DIM, 3><<<nblocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_, ch);
    return check_launch();
  }
}

#define PMG_DISPATCH(dtype, dim, CALL)                  \
  do {                                                  \
    if ((dtype) == PMG_F64 && (dim) == 3) {             \
      using T = double;                                 \
      constexpr int DIM = 3;                            \
      return CALL;                                      \
    } else if ((dtype) == PMG_F64) {                    \
      using T = double;                                 \
      constexpr int DIM = 2;                            \
      return CALL;                                      \
    } else if ((dim) == 3) {                            \
      using T = float;                                  \
      constexpr int DIM = 3;                            \
      return CALL;                                      \
    } else {                                            \
      using T = float;                                  \
      constexpr int DIM = 2;                            \
      return CALL;                                      \
    }                                                   \
  } while (0)

// Thread per (node = x index, stored stencil offset = blockIdx.y).
template <typename T, int DIM, typename Kern, typename... Args>
int launch_per_stored_offset(Kern kernel, const Grid& g, cudaStream_t st, Args... args) {
  const dim3 grid(blocks_for(g.nnodes(), 256), Traits<DIM>::NH);
  kernel<<<grid, 256, 0, st>>>(args...);
  return check_launch();
}

template <typename T, int DIM, typename Kern, typename... Args>
int launch_simple(Kern kernel, int64_t n, cudaStream_t st, Args... args) {
  if (n <= 0) return PMG_OK;
  const int threads = 256;
  kernel<<<blocks_for(n, threads), threads, 0, st>>>(args...);
  return check_launch();
}

}  // namespace pmg

using namespace pmg;

static bool dtype_ok(int dtype) { return dtype == PMG_F64 || dtype == PMG_F32; }

// A multiplier coprime to n (visiting i -> i * m mod n is then a permutation of 0..n-1).
static unsigned coprime_stride(int64_t n) {
  const unsigned cands[] = {10007u, 10009u, 10037u, 1009u, 101u, 7u};
  for (unsigned m : cands) {
    int64_t a = n, b = m;
    while (b) {
      const int64_t t = a % b;
      a = b;
      b = t;
    }
    if (a == 1) return m;
  }
  return 1u;
}

extern "C" {

int pmg_dof_connectivity(int nelx, int nely, int nelz, int64_t* dofconn, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dofconn) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  dofconn_kernel<<<blocks_for(g.nel(), 256), 256, 0, as_stream(stream)>>>(g, dofconn);
  return check_launch();
}

int pmg_ebe_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                  const uint8_t* bcmask, double bcdiag, const void* u, const void* b, const void* diag,
                  double omega, void* y, const void* cdiag, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !xe || !K0_host || !u || !y) return PMG_BAD_ARG;
  if (mode < 0 || mode > 2) return PMG_BAD_ARG;
  if (mode >= PMG_APPLY_RESIDUAL && !b) return PMG_BAD_ARG;
  if (mode == PMG_APPLY_JACOBI && !diag) return PMG_BAD_ARG;
  if (y == u) return PMG_BAD_ARG;  // the gather reads the neighbourhood of u
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (ebe_apply_t<T, DIM>(mode, g, xe, K0_host, bcmask, bcdiag, u, b, diag, omega, y, cdiag,
                                    as_stream(stream))));
}

int pmg_ebe_diagonal(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                     const uint8_t* bcmask, double bcdiag, void* diag, const void* cdiag, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !xe || !K0_host || !diag) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(ebe_diag_kernel<T, DIM>, g.nnodes(), as_stream(stream), g, (const T*)xe,
                                      make_elem_mat<T, Traits<DIM>::NDE>(K0_host), bcmask, (T)bcdiag, (T*)diag,
                                      (const T*)cdiag)));
}

int pmg_stencil_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* S, const void* u,
                      const void* b, const void* diag, double omega, void* y, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !u || !y || y == u) return PMG_BAD_ARG;
  if (mode < 0 || mode > 2) return PMG_BAD_ARG;
  if (mode >= PMG_APPLY_RESIDUAL && !b) return PMG_BAD_ARG;
  if (mode == PMG_APPLY_JACOBI && !diag) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(), (stencil_apply_t<T, DIM>(mode, g, S, u, b, diag, omega, y, as_stream(stream))));
}

int pmg_stencil_cheb_step(int dtype, int nelx, int nely, int nelz, const void* S, const void* u, const void* b,
                          const void* dl1, void* d, const double* coef, int step, void* y, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !u || !b || !dl1 || !d || !coef || !y || y == u ||
      step < 0 || step >= 64)
    return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (stencil_apply_t<T, DIM>(PMG_APPLY_CHEB, g, S, u, b, dl1, 0.0, y, as_stream(stream),
                                        ChebArgs<T>{(T*)d, coef, step})));
}

int pmg_ebe_cheb_step(int nelx, int nely, int nelz, const float* xe, const double* K0_host, const uint8_t* bcmask,
                      double bcdiag, const float* u, const float* b, const float* dl1, float* d, const double* coef,
                      int step, float* y, const float* cdiag, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || nelz == 0 || !xe || !K0_host || !u || !b || !dl1 || !d || !coef || !y || y == u ||
      step < 0 || step >= 64)
    return PMG_BAD_ARG;
  return ebe_apply_f32_3d(PMG_APPLY_CHEB, Grid{nelx, nely, nelz}, xe, K0_host, bcmask, bcdiag, u, b, dl1, 0.0, y,
                          ChebArgs<float>{d, coef, step}, cdiag, as_stream(stream));
}

int pmg_set_operator_kernel(int kind) {
  if (kind == -1) return pmg::g_f32_operator.load();
  if (kind != PMG_OPERATOR_FMA && kind != PMG_OPERATOR_TCGEN05) return -1;
  return pmg::g_f32_operator.exchange(kind);
}

int pmg_stencil_add_diagonal(int dtype, int nelx, int nely, int nelz, void* S, const void* c, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !c) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(stencil_add_diag_kernel<T, DIM>, g.nnodes(), as_stream(stream), g, (T*)S,
                                      (const T*)c)));
}

int pmg_stencil_diagonal(int dtype, int nelx, int nely, int nelz, const void* S, void* diag, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !diag) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(stencil_diag_kernel<T, DIM>, g.nnodes(), as_stream(stream), g, (const T*)S,
                                      (T*)diag)));
}

int pmg_stencil_rowabs(int dtype, int nelx, int nely, int nelz, const void* S, void* out, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !out) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(stencil_rowabs_kernel<T, DIM>, g.nnodes() * DIM, as_stream(stream), g,
                                      (const T*)S, (T*)out)));
}

static bool even_grid(int nx, int ny, int nz) { return nx % 2 == 0 && ny % 2 == 0 && nz % 2 == 0 && nx >= 2 && ny >= 2; }

int pmg_restrict(int dtype, int nelx, int nely, int nelz, const void* rf, void* rc, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !even_grid(nelx, nely, nelz) || !rf || !rc) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(restrict_kernel<T, DIM>, g.coarse().nnodes(), as_stream(stream), g,
                                      (const T*)rf, (T*)rc)));
}

int pmg_prolong_add(int dtype, int nelx, int nely, int nelz, const void* uc, void* uf, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !even_grid(nelx, nely, nelz) || !uc || !uf) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(prolong_add_kernel<T, DIM>, g.nnodes(), as_stream(stream), g,
                                      (const T*)uc, (T*)uf)));
}

int pmg_galerkin_table(int dim, const double* K0, double* table) {
  if ((dim != 2 && dim != 3) || !K0 || !table) return PMG_BAD_ARG;
  const int nn = 1 << dim, nde = nn * dim;
  // M_s[(a,d),(A,e)] = delta_de * prod_axis p1(s_axis, a_axis, A_axis)
  auto M = [&](int s, int qa, int qA) -> double {
    const int a = qa / dim, d = qa % dim, A = qA / dim, e = qA % dim;
    if (d != e) return 0.0;
    double w = 1.0;
    for (int ax = 0; ax < dim; ++ax) w *= p1((s >> ax) & 1, (a >> ax) & 1, (A >> ax) & 1);
    return w;
  };
  for (int s = 0; s < nn; ++s) {
    for (int r = 0; r < nde; ++r)
      for (int c = 0; c < nde; ++c) {
        double v = 0.0;
        for (int p = 0; p < nde; ++p) {
          const double mpr = M(s, p, r);
          if (mpr == 0.0) continue;
          for (int q = 0; q < nde; ++q) {
            const double mqc = M(s, q, c);
            if (mqc != 0.0) v += mpr * K0[p * nde + q] * mqc;
          }
        }
        table[(size_t)s * nde * nde + r * nde + c] = v;
      }
  }
  return PMG_OK;
}

int pmg_galerkin_from_ebe(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                          const uint8_t* bcmask, double bcdiag, const void* table, const int32_t* bc_elems, int n_bc,
                          void* Ec, void* stream) {
  if (n_bc < 0 || (n_bc > 0 && !bc_elems)) return PMG_BAD_ARG;
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !even_grid(nelx, nely, nelz) || !xe || !K0_host || !table ||
      !Ec)
    return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const int64_t nelc = g.coarse().nel();
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned nblk = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nelc + GAL_WARPS - 1) / GAL_WARPS, 4 * sms));
  cudaStream_t st = as_stream(stream);
  PMG_DISPATCH(dtype, g.dim(), ([&]() -> int {
                 constexpr int NE = Traits<DIM>::NDE * Traits<DIM>::NDE;
                 const size_t smem = sizeof(T) * (size_t)(Traits<DIM>::NN + 4) * NE;
                 cudaError_t e = cudaFuncSetAttribute(galerkin_from_ebe_kernel<T, DIM>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                 if (e != cudaSuccess) {
                   set_error(cudaGetErrorString(e));
                   return PMG_CUDA_ERR;
                 }
                 const auto K = make_elem_mat<T, Traits<DIM>::NDE>(K0_host);
                 galerkin_from_ebe_kernel<T, DIM><<<nblk, GAL_THREADS, smem, st>>>(
                     g, (const T*)xe, K, bcmask, (T)bcdiag, (const T*)table, (T*)Ec, coprime_stride(nelc),
                     bc_elems != nullptr);
                 if (bc_elems && n_bc > 0) {
                   const size_t smem2 = sizeof(T) * 4 * (size_t)NE;
                   e = cudaFuncSetAttribute(galerkin_listed_kernel<T, DIM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem2);
                   if (e != cudaSuccess) {
                     set_error(cudaGetErrorString(e));
                     return PMG_CUDA_ERR;
                   }
                   galerkin_listed_kernel<T, DIM><<<n_bc, GAL_THREADS, smem2, st>>>(g, (const T*)xe, K, bcmask, (T)bcdiag,
                                                                                    (const T*)table, bc_elems, (T*)Ec);
                 }
                 return check_launch();
               }()));
}

int pmg_galerkin_from_elements(int dtype, int nelx, int nely, int nelz, const void* Ef, void* Ec, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !even_grid(nelx, nely, nelz) || !Ef || !Ec) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const int64_t nelc = g.coarse().nel();
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned nblk = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nelc + GAL_WARPS - 1) / GAL_WARPS, 8 * sms));
  cudaStream_t st = as_stream(stream);
  PMG_DISPATCH(dtype, g.dim(), ([&]() -> int {
                 constexpr int NDE = Traits<DIM>::NDE;
                 const size_t smem = sizeof(T) * GAL_WARPS * (size_t)(NDE * (NDE + 1) + NDE * NDE);
                 cudaError_t e = cudaFuncSetAttribute(galerkin_from_elements_kernel<T, DIM>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                 if (e != cudaSuccess) {
                   set_error(cudaGetErrorString(e));
                   return PMG_CUDA_ERR;
                 }
                 galerkin_from_elements_kernel<T, DIM><<<nblk, GAL_THREADS, smem, st>>>(g, (const T*)Ef, (T*)Ec);
                 return check_launch();
               }()));
}

int pmg_stencil_from_elements(int dtype, int nelx, int nely, int nelz, const void* E, void* S, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !E || !S) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_per_stored_offset<T, DIM>(stencil_from_elements_kernel<T, DIM>, g, as_stream(stream), g,
                                                 (const T*)E, (T*)S)));
}

int pmg_ebe_stencil(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                    const uint8_t* bcmask, double bcdiag, void* S, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !xe || !K0_host || !S) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_per_stored_offset<T, DIM>(ebe_stencil_kernel<T, DIM>, g, as_stream(stream), g, (const T*)xe,
                                                 make_elem_mat<T, Traits<DIM>::NDE>(K0_host), bcmask, (T)bcdiag,
                                                 (T*)S)));
}

int pmg_stencil_to_dense(int dtype, int nelx, int nely, int nelz, const void* S, double* A, void* stream) {
  return pmg_stencil_to_dense_perm(dtype, nelx, nely, nelz, S, nullptr, A, stream);
}

int pmg_stencil_to_dense_perm(int dtype, int nelx, int nely, int nelz, const void* S, const int32_t* pos, double* A,
                              void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !A) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const int64_t ndof = g.nnodes() * g.dim();
  if (ndof > 65536) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  cudaError_t e = cudaMemsetAsync(A, 0, sizeof(double) * ndof * ndof, st);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  PMG_DISPATCH(dtype, g.dim(),
               (launch_per_stored_offset<T, DIM>(stencil_to_dense_kernel<T, DIM>, g, st, g, (const T*)S, pos, A)));
}

int pmg_coarse_ordering(int nelx, int nely, int nelz, int32_t* pos, int* bw) {
  if (!grid_ok(nelx, nely, nelz) || !pos || !bw) return PMG_BAD_ARG;
  const int dim = nelz == 0 ? 2 : 3;
  const int cnt[3] = {nelx + 1, nely + 1, dim == 3 ? nelz + 1 : 1};
  // axes by node count, fewest first (fastest): a band of (count0 * count1 + count0 + 1) nodes
  int ax[3] = {0, 1, 2};
  for (int a = 0; a < dim; ++a)
    for (int b = a + 1; b < dim; ++b)
      if (cnt[ax[b]] < cnt[ax[a]]) std::swap(ax[a], ax[b]);
  const int c0 = cnt[ax[0]], c1 = cnt[ax[1]];
  int idx[3];
  for (idx[2] = 0; idx[2] < cnt[2]; ++idx[2])
    for (idx[1] = 0; idx[1] < cnt[1]; ++idx[1])
      for (idx[0] = 0; idx[0] < cnt[0]; ++idx[0]) {
        const int64_t nat = ((int64_t)idx[2] * cnt[1] + idx[1]) * cnt[0] + idx[0];
        const int64_t p = dim == 3 ? ((int64_t)idx[ax[2]] * c1 + idx[ax[1]]) * c0 + idx[ax[0]]
                                   : (int64_t)idx[ax[1]] * c0 + idx[ax[0]];
        for (int d = 0; d < dim; ++d) pos[nat * dim + d] = (int32_t)(p * dim + d);
      }
  const int64_t dn = 1 + c0 + (dim == 3 ? (int64_t)c0 * c1 : 0);
  *bw = (int)(dn * dim + dim - 1);
  return PMG_OK;
}

int pmg_stencil_bandwidth(int nelx, int nely, int nelz) {
  if (!grid_ok(nelx, nely, nelz)) return -1;
  const int dim = nelz == 0 ? 2 : 3;
  // farthest coupled node: offset (1,1,1) -> node distance 1 + nnx + nnx*nny
  const int64_t dn = 1 + (int64_t)(nelx + 1) + (dim == 3 ? (int64_t)(nelx + 1) * (nely + 1) : 0);
  return (int)(dn * dim + dim - 1);
}

}  // extern "C"
