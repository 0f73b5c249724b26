// Stiffness operators of the multigrid hierarchy.
//
//  level 0: matrix-free K(x) u = sum_e x_e K0 u_e with Dirichlet rows/cols (node-centric gather: every
//           thread owns one node, reads the 3^dim neighbourhood of u once into registers and sums the
//           2^dim element contributions; no atomics, deterministic).
//  level>0: assembled node stencils (3^dim blocks of dim x dim per node, structure-of-arrays).
//  transfers: trilinear restriction / prolongation as gathers.
//  Galerkin: coarse element matrices E_C = sum_c M_c^T E_c M_c by sum factorisation.
#include <cstdio>

#include "common.cuh"

namespace pmg {

// ------------------------------------------------------------------------------------------ level 0
// MODE 0: y = K u;  1: y = b - K u;  2: y = u + w * ((b - K u) / diag)
template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(128) ebe_apply_kernel(Grid g, const T* __restrict__ xe, ElemMat<T, Traits<DIM>::NDE> K0,
                                                        const uint8_t* __restrict__ bcmask, T bcdiag,
                                                        const T* __restrict__ u, const T* __restrict__ b,
                                                        const T* __restrict__ diag, T w, T* __restrict__ y) {
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
    if (MODE == 0) {
      y[q] = Au;
    } else if (MODE == 1) {
      y[q] = b[q] - Au;
    } else {
      y[q] = u[q] + w * ((b[q] - Au) / diag[q]);
    }
  }
}

template <typename T, int DIM>
__global__ void ebe_diag_kernel(Grid g, const T* __restrict__ xe, ElemMat<T, Traits<DIM>::NDE> K0,
                                const uint8_t* __restrict__ bcmask, T bcdiag, T* __restrict__ diag) {
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
  for (int d = 0; d < DIM; ++d) diag[n * DIM + d] = ((m >> d) & 1) ? bcdiag : acc[d];
}

// ------------------------------------------------------------------------------------------ stencils
template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(128) stencil_apply_kernel(Grid g, const T* __restrict__ S, const T* __restrict__ u,
                                                            const T* __restrict__ b, const T* __restrict__ diag, T w,
                                                            T* __restrict__ y) {
  constexpr int NOFF = Traits<DIM>::NOFF;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  T acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = T(0);
#pragma unroll
  for (int o = 0; o < NOFF; ++o) {
    const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = DIM == 3 ? o / 9 - 1 : 0;
    const int ii = i + dx, jj = j + dy, kk = k + dz;
    if (ii < 0 || ii > g.nx || jj < 0 || jj > g.ny || kk < 0 || kk > g.nz) continue;
    const int64_t m = node_id(g, ii, jj, kk);
    T um[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) um[c] = u[m * DIM + c];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int c = 0; c < DIM; ++c) acc[d] = fma(S[((int64_t)(o * DIM + d) * DIM + c) * nn + n], um[c], acc[d]);
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const int64_t q = n * DIM + d;
    if (MODE == 0) {
      y[q] = acc[d];
    } else if (MODE == 1) {
      y[q] = b[q] - acc[d];
    } else {
      y[q] = u[q] + w * ((b[q] - acc[d]) / diag[q]);
    }
  }
}

template <typename T, int DIM>
__global__ void stencil_diag_kernel(Grid g, const T* __restrict__ S, T* __restrict__ diag) {
  constexpr int C = DIM == 3 ? 13 : 4;
  const int64_t nn = g.nnodes();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
#pragma unroll
  for (int d = 0; d < DIM; ++d) diag[n * DIM + d] = S[((int64_t)(C * DIM + d) * DIM + d) * nn + n];
}

// ------------------------------------------------------------------------------------------ transfers
// weight of a fine node at signed offset a (in fine units) from a coarse node: 1 at 0, 1/2 at +-1
__device__ __forceinline__ double tw(int a) { return a == 0 ? 1.0 : 0.5; }

// rc = R^T rf, one thread per coarse node (gather over the 3^dim fine neighbourhood)
template <typename T, int DIM>
__global__ void restrict_kernel(Grid gf, const T* __restrict__ rf, T* __restrict__ rc) {
  const Grid gc = gf.coarse();
  const int64_t N = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (N >= gc.nnodes()) return;
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
        if (i < 0 || i > gf.nx || j < 0 || j > gf.ny || k < 0 || k > gf.nz) continue;
        const T wgt = (T)(tw(a) * tw(bb) * tw(c));
        const int64_t m = node_id(gf, i, j, k);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = fma(wgt, rf[m * DIM + d], acc[d]);
      }
#pragma unroll
  for (int d = 0; d < DIM; ++d) rc[N * DIM + d] = acc[d];
}

// uf += R uc, one thread per fine node (gather over the <= 2^dim coarse parents)
template <typename T, int DIM>
__global__ void prolong_add_kernel(Grid gf, const T* __restrict__ uc, T* __restrict__ uf) {
  const Grid gc = gf.coarse();
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= gf.nnodes()) return;
  int i, j, k;
  node_ijk(gf, n, i, j, k);
  T acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = T(0);
  const int i0 = i >> 1, j0 = j >> 1, k0 = k >> 1;
  const int ni = (i & 1) + 1, nj = (j & 1) + 1, nk = (DIM == 3) ? (k & 1) + 1 : 1;
  for (int c = 0; c < nk; ++c)
    for (int bb = 0; bb < nj; ++bb)
      for (int a = 0; a < ni; ++a) {
        const T wgt = (T)((ni == 2 ? 0.5 : 1.0) * (nj == 2 ? 0.5 : 1.0) * (nk == 2 ? 0.5 : 1.0));
        const int64_t M = node_id(gc, i0 + a, j0 + bb, k0 + c);
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = fma(wgt, uc[M * DIM + d], acc[d]);
      }
#pragma unroll
  for (int d = 0; d < DIM; ++d) uf[n * DIM + d] += acc[d];
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
// One CTA per coarse element.  Unconstrained children use the precomputed table; children touching a
// Dirichlet dof are transformed explicitly with their masked matrix plus the bcdiag terms of the fine
// Dirichlet dofs assigned to them (each fine node is assigned to the element min(i, nx-1), ...).
template <typename T, int DIM>
__global__ void galerkin_from_ebe_kernel(Grid gf, const T* __restrict__ xe, ElemMat<T, Traits<DIM>::NDE> K0,
                                         const uint8_t* __restrict__ bcmask, T bcdiag, const T* __restrict__ table,
                                         T* __restrict__ Ec) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  __shared__ T E[NE];
  __shared__ T Kc[NE];
  __shared__ T buf[NE];
  __shared__ uint8_t cmask[NN];
  __shared__ int any_bc;
  const Grid gc = gf.coarse();
  const int64_t ec = blockIdx.x;
  const int CI = (int)(ec % gc.nx), CJ = (int)((ec / gc.nx) % gc.ny), CK = (int)(ec / ((int64_t)gc.nx * gc.ny));
  for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] = T(0);
  __syncthreads();
  for (int s = 0; s < NN; ++s) {
    const int fi = 2 * CI + (s & 1), fj = 2 * CJ + ((s >> 1) & 1), fk = DIM == 3 ? 2 * CK + ((s >> 2) & 1) : 0;
    const T x = xe[elem_id(gf, fi, fj, fk)];
    if (threadIdx.x == 0) any_bc = 0;
    __syncthreads();
    if (threadIdx.x < NN) {
      const int a = threadIdx.x;
      const int ni = fi + (a & 1), nj = fj + ((a >> 1) & 1), nk = DIM == 3 ? fk + ((a >> 2) & 1) : 0;
      const uint8_t m = bcmask ? bcmask[node_id(gf, ni, nj, nk)] : 0;
      cmask[a] = m;
      if (m) atomicOr(&any_bc, 1);
    }
    __syncthreads();
    if (!any_bc) {
      for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] = fma(x, table[s * NE + e], E[e]);
      __syncthreads();
      continue;
    }
    // masked child matrix x Z K0 Z + bcdiag on assigned Dirichlet dofs
    for (int e = threadIdx.x; e < NE; e += blockDim.x) {
      const int r = e / NDE, c = e % NDE;
      const int rn = r / DIM, rd = r % DIM, cn = c / DIM, cd = c % DIM;
      const bool rb = (cmask[rn] >> rd) & 1, cb = (cmask[cn] >> cd) & 1;
      T v = (rb || cb) ? T(0) : x * K0.v[e];
      if (r == c && rb) {
        // assigned to this fine element?
        const int ni = fi + (rn & 1), nj = fj + ((rn >> 1) & 1), nk = DIM == 3 ? fk + ((rn >> 2) & 1) : 0;
        const int ai = min(ni, gf.nx - 1), aj = min(nj, gf.ny - 1), ak = DIM == 3 ? min(nk, gf.nz - 1) : 0;
        if (ai == fi && aj == fj && ak == fk) v = bcdiag;
      }
      Kc[e] = v;
    }
    __syncthreads();
    galerkin_child_accumulate<T, DIM>(E, Kc, buf, s);
  }
  for (int e = threadIdx.x; e < NE; e += blockDim.x) Ec[ec * NE + e] = E[e];
}

// Next-level coarse element matrices from element matrices Ef of grid gf.
template <typename T, int DIM>
__global__ void galerkin_from_elements_kernel(Grid gf, const T* __restrict__ Ef, T* __restrict__ Ec) {
  constexpr int NN = Traits<DIM>::NN;
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  __shared__ T E[NE];
  __shared__ T Kc[NE];
  __shared__ T buf[NE];
  const Grid gc = gf.coarse();
  const int64_t ec = blockIdx.x;
  const int CI = (int)(ec % gc.nx), CJ = (int)((ec / gc.nx) % gc.ny), CK = (int)(ec / ((int64_t)gc.nx * gc.ny));
  for (int e = threadIdx.x; e < NE; e += blockDim.x) E[e] = T(0);
  __syncthreads();
  for (int s = 0; s < NN; ++s) {
    const int fi = 2 * CI + (s & 1), fj = 2 * CJ + ((s >> 1) & 1), fk = DIM == 3 ? 2 * CK + ((s >> 2) & 1) : 0;
    const T* src = Ef + elem_id(gf, fi, fj, fk) * NE;
    for (int e = threadIdx.x; e < NE; e += blockDim.x) Kc[e] = src[e];
    __syncthreads();
    galerkin_child_accumulate<T, DIM>(E, Kc, buf, s);
  }
  for (int e = threadIdx.x; e < NE; e += blockDim.x) Ec[ec * NE + e] = E[e];
}

// Node stencils from element matrices: thread per (offset o, node n).
template <typename T, int DIM>
__global__ void stencil_from_elements_kernel(Grid g, const T* __restrict__ E, T* __restrict__ S) {
  constexpr int NDE = Traits<DIM>::NDE;
  constexpr int NE = NDE * NDE;
  constexpr int NOFF = Traits<DIM>::NOFF;
  const int64_t nn = g.nnodes();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn * NOFF) return;
  const int o = (int)(t / nn);
  const int64_t n = t % nn;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = DIM == 3 ? o / 9 - 1 : 0;
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
    for (int c = 0; c < DIM; ++c) S[((int64_t)(o * DIM + d) * DIM + c) * nn + n] = acc[d * DIM + c];
}

template <typename T, int DIM>
__global__ void stencil_to_dense_kernel(Grid g, const T* __restrict__ S, double* __restrict__ A) {
  constexpr int NOFF = Traits<DIM>::NOFF;
  const int64_t nn = g.nnodes();
  const int64_t ndof = nn * DIM;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn * NOFF) return;
  const int o = (int)(t / nn);
  const int64_t n = t % nn;
  int i, j, k;
  node_ijk(g, n, i, j, k);
  const int ii = i + o % 3 - 1, jj = j + (o / 3) % 3 - 1, kk = k + (DIM == 3 ? o / 9 - 1 : 0);
  if (ii < 0 || ii > g.nx || jj < 0 || jj > g.ny || kk < 0 || kk > g.nz) return;
  const int64_t m = node_id(g, ii, jj, kk);
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int c = 0; c < DIM; ++c)
      A[(n * DIM + d) * ndof + m * DIM + c] = (double)S[((int64_t)(o * DIM + d) * DIM + c) * nn + n];
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
template <typename T, int DIM>
int ebe_apply_t(int mode, Grid g, const void* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                const void* u, const void* b, const void* diag, double w, void* y, cudaStream_t st) {
  auto K = make_elem_mat<T, Traits<DIM>::NDE>(K0);
  const int threads = 128;
  const unsigned blocks = blocks_for(g.nnodes(), threads);
  const T* xe_ = (const T*)xe;
  const T* u_ = (const T*)u;
  const T* b_ = (const T*)b;
  const T* d_ = (const T*)diag;
  T* y_ = (T*)y;
  if (mode == PMG_APPLY_MATVEC)
    ebe_apply_kernel<T, DIM, 0><<<blocks, threads, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_);
  else if (mode == PMG_APPLY_RESIDUAL)
    ebe_apply_kernel<T, DIM, 1><<<blocks, threads, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_);
  else
    ebe_apply_kernel<T, DIM, 2><<<blocks, threads, 0, st>>>(g, xe_, K, bcmask, (T)bcdiag, u_, b_, d_, (T)w, y_);
  return check_launch();
}

template <typename T, int DIM>
int stencil_apply_t(int mode, Grid g, const void* S, const void* u, const void* b, const void* diag, double w,
                    void* y, cudaStream_t st) {
  const int threads = 128;
  const unsigned blocks = blocks_for(g.nnodes(), threads);
  const T* S_ = (const T*)S;
  const T* u_ = (const T*)u;
  const T* b_ = (const T*)b;
  const T* d_ = (const T*)diag;
  T* y_ = (T*)y;
  if (mode == PMG_APPLY_MATVEC)
    stencil_apply_kernel<T, DIM, 0><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_);
  else if (mode == PMG_APPLY_RESIDUAL)
    stencil_apply_kernel<T, DIM, 1><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_);
  else
    stencil_apply_kernel<T, DIM, 2><<<blocks, threads, 0, st>>>(g, S_, u_, b_, d_, (T)w, y_);
  return check_launch();
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

extern "C" {

int pmg_dof_connectivity(int nelx, int nely, int nelz, int64_t* dofconn, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dofconn) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  dofconn_kernel<<<blocks_for(g.nel(), 256), 256, 0, as_stream(stream)>>>(g, dofconn);
  return check_launch();
}

int pmg_ebe_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                  const uint8_t* bcmask, double bcdiag, const void* u, const void* b, const void* diag,
                  double omega, void* y, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !xe || !K0_host || !u || !y) return PMG_BAD_ARG;
  if (mode < 0 || mode > 2) return PMG_BAD_ARG;
  if (mode >= PMG_APPLY_RESIDUAL && !b) return PMG_BAD_ARG;
  if (mode == PMG_APPLY_JACOBI && !diag) return PMG_BAD_ARG;
  if (y == u) return PMG_BAD_ARG;  // the gather reads the neighbourhood of u
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (ebe_apply_t<T, DIM>(mode, g, xe, K0_host, bcmask, bcdiag, u, b, diag, omega, y, as_stream(stream))));
}

int pmg_ebe_diagonal(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                     const uint8_t* bcmask, double bcdiag, void* diag, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !xe || !K0_host || !diag) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(ebe_diag_kernel<T, DIM>, g.nnodes(), as_stream(stream), g, (const T*)xe,
                                      make_elem_mat<T, Traits<DIM>::NDE>(K0_host), bcmask, (T)bcdiag, (T*)diag)));
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

int pmg_stencil_diagonal(int dtype, int nelx, int nely, int nelz, const void* S, void* diag, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !S || !diag) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(stencil_diag_kernel<T, DIM>, g.nnodes(), as_stream(stream), g, (const T*)S,
                                      (T*)diag)));
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
               (launch_simple<T, DIM>(prolong_add_kernel<T, DIM>, g.nnodes(), as_stream(stream), g, (const T*)uc,
                                      (T*)uf)));
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
                          const uint8_t* bcmask, double bcdiag, const void* table, void* Ec, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !even_grid(nelx, nely, nelz) || !xe || !K0_host || !table ||
      !Ec)
    return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const unsigned nblk = (unsigned)g.coarse().nel();
  const int threads = g.dim() == 3 ? 288 : 64;
  cudaStream_t st = as_stream(stream);
  PMG_DISPATCH(dtype, g.dim(), ([&]() -> int {
                 galerkin_from_ebe_kernel<T, DIM><<<nblk, threads, 0, st>>>(
                     g, (const T*)xe, make_elem_mat<T, Traits<DIM>::NDE>(K0_host), bcmask, (T)bcdiag, (const T*)table,
                     (T*)Ec);
                 return check_launch();
               }()));
}

int pmg_galerkin_from_elements(int dtype, int nelx, int nely, int nelz, const void* Ef, void* Ec, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !even_grid(nelx, nely, nelz) || !Ef || !Ec) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const unsigned nblk = (unsigned)g.coarse().nel();
  const int threads = g.dim() == 3 ? 288 : 64;
  cudaStream_t st = as_stream(stream);
  PMG_DISPATCH(dtype, g.dim(), ([&]() -> int {
                 galerkin_from_elements_kernel<T, DIM><<<nblk, threads, 0, st>>>(g, (const T*)Ef, (T*)Ec);
                 return check_launch();
               }()));
}

int pmg_stencil_from_elements(int dtype, int nelx, int nely, int nelz, const void* E, void* S, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || !dtype_ok(dtype) || !E || !S) return PMG_BAD_ARG;
  Grid g{nelx, nely, nelz};
  const int64_t work = g.nnodes() * (g.dim() == 3 ? 27 : 9);
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(stencil_from_elements_kernel<T, DIM>, work, as_stream(stream), g, (const T*)E,
                                      (T*)S)));
}

int pmg_stencil_to_dense(int dtype, int nelx, int nely, int nelz, const void* S, double* A, void* stream) {
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
  const int64_t work = g.nnodes() * (g.dim() == 3 ? 27 : 9);
  PMG_DISPATCH(dtype, g.dim(),
               (launch_simple<T, DIM>(stencil_to_dense_kernel<T, DIM>, work, st, g, (const T*)S, A)));
}

int pmg_stencil_bandwidth(int nelx, int nely, int nelz) {
  if (!grid_ok(nelx, nely, nelz)) return -1;
  const int dim = nelz == 0 ? 2 : 3;
  // farthest coupled node: offset (1,1,1) -> node distance 1 + nnx + nnx*nny
  const int64_t dn = 1 + (int64_t)(nelx + 1) + (dim == 3 ? (int64_t)(nelx + 1) * (nely + 1) : 0);
  return (int)(dn * dim + dim - 1);
}

}  // extern "C"
