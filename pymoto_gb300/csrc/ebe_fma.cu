// Matrix-free hex8 operator (FP32) on the CUDA cores: one thread per node column, walking up the z layers.
//
// K(x) u = sum_e x_e K0 u_e (pymoto/modules/assembly.py:245-296 assembles the same sum as a CSR matrix).
//
// Work split.  A CTA owns a tile of OX x OY node columns (OX, OY chosen per grid so that the tiles cover the
// node counts with little waste; OX <= 32, OY <= 32, OX OY <= 256) and a chunk of node layers; thread t owns
// column (t mod OX, t div OX) of the tile.  For element layer k (between node layers k and k + 1) the thread
// takes the 4 elements of the layer around its column and, per element, the 3 rows of K0 of its node on the
// lower face and the 3 rows of its node on the upper face (4 x 6 x 24 = 576 FMAs per node, K0 read from the
// kernel parameters as a uniform operand).  The lower-face rows complete node k together with the upper-face
// rows of element layer k - 1, which the thread carried in registers; the upper-face rows are carried to node
// k + 1.  Every node is summed by its own thread in a fixed order: no atomics, deterministic results, and no
// element product is computed twice.
//
// Staging.  Node layers of u (constrained dofs zeroed, then shifted by one displacement of the tile: K0
// annihilates a common translation of an element's nodes, so the rounding error scales with the variation of
// u over the tile, not with |u|), their constraint-mask words and the element layers of x are copied with
// cp.async two layers ahead into a 4-slot ring.  One CTA barrier per layer.
//
// Cube elements.  The element matrix of an isotropic cube element has 10 distinct entries up to a sign that
// does not depend on the material (hex8_classes.cuh); for such a K0 the kernel is instantiated with the 10
// values as kernel parameters and the class and sign of every entry as compile-time constants, so each FMA takes
// one of 10 uniform operands instead of one of 576 (measured: 13 % fewer instructions, 13 % less time).  Other
// element matrices use the general instantiation.
#include "common.cuh"
#include "hex8_classes.cuh"

#include <algorithm>
#include <cmath>

namespace pmg {
namespace {

constexpr int FT = 256;                 // threads per CTA
constexpr int FPLANE_MAX = 340;         // staged nodes per layer: (OX + 2)(OY + 2) <= 340 under the tile limits
constexpr int FEPLANE_MAX = 297;        // staged elements per layer: (OX + 1)(OY + 1) <= 297
constexpr int FRING = 4;                // node layers t, t + 1 in use, t + 2 and t + 3 in flight
constexpr int FPN = (FPLANE_MAX + FT - 1) / FT;
constexpr int FPE = (FEPLANE_MAX + FT - 1) / FT;

struct FmaSmem {
  float4 u[FRING][FPLANE_MAX];          // (ux, uy, uz, 0) of the staged nodes
  uint32_t m[FRING][FPLANE_MAX];        // aligned bcmask word holding each staged node's mask byte
  float x[FRING][FEPLANE_MAX];          // element layer of x
};

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
               "l"(gmem), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ float comp(const float4& v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }

struct CubeVals {
  float v[HEX8_CLASSES];
};

// Entry i of K0: from the parameters, or for a cube element from its class value and sign.
template <bool CUBE>
__device__ __forceinline__ float k0(const ElemMat<float, 24>& K0, const CubeVals& cv, int i) {
  if (CUBE) return K0_SIGN[i] > 0 ? cv.v[K0_CLASS[i]] : -cv.v[K0_CLASS[i]];
  return K0.v[i];
}

// Forces of element layer k on the thread's node column: lower-face rows into ab (node layer k), upper-face
// rows into at (node layer k + 1).  ub / ut: the staged node layers k, k + 1 at the corner of the column's
// 3 x 3 window (row length NX); xv: x of the 4 elements around the column.  The loop runs over the 18 window
// nodes and adds each to the elements that hold it, so only one node and the 24 element sums are live.
template <bool BOT, bool TOP, bool CUBE>
__device__ __forceinline__ void element_layer(const ElemMat<float, 24>& K0, const CubeVals& cv, const float4* ub,
                                              const float4* ut, int NX, const float (&xv)[4], float (&ab)[3],
                                              float (&at)[3]) {
  float tb[4][3], tt[4][3];
#pragma unroll
  for (int e = 0; e < 4; ++e)
#pragma unroll
    for (int d = 0; d < 3; ++d) tb[e][d] = tt[e][d] = 0.f;
#pragma unroll
  for (int wz = 0; wz < 2; ++wz)
#pragma unroll
    for (int wy = 0; wy < 3; ++wy)
#pragma unroll
      for (int wx = 0; wx < 3; ++wx) {
        const float4 v = (wz ? ut : ub)[wy * NX + wx];
#pragma unroll
        for (int oy = 0; oy < 2; ++oy)
#pragma unroll
          for (int ox = 0; ox < 2; ++ox) {
            const int lx = wx - ox, ly = wy - oy;
            if (lx < 0 || lx > 1 || ly < 0 || ly > 1) continue;
            const int e = oy * 2 + ox;
            const int lb = lx + 2 * ly + 4 * wz;        // the window node in the element
            const int ln = (1 - ox) + 2 * (1 - oy);     // the column's node on the element's lower face
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float uc = comp(v, c);
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                if (BOT) tb[e][d] = fmaf(k0<CUBE>(K0, cv, (ln * 3 + d) * 24 + lb * 3 + c), uc, tb[e][d]);
                if (TOP) tt[e][d] = fmaf(k0<CUBE>(K0, cv, ((ln + 4) * 3 + d) * 24 + lb * 3 + c), uc, tt[e][d]);
              }
            }
          }
      }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ab[d] = at[d] = 0.f;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (BOT) ab[d] = fmaf(xv[e], tb[e][d], ab[d]);
      if (TOP) at[d] = fmaf(xv[e], tt[e][d], at[d]);
    }
  }
}

template <int MODE, bool CUBE>
__global__ void __launch_bounds__(FT, 2)
    ebe_apply_fma_kernel(Grid g, int OX, int OY, const float* __restrict__ xe, ElemMat<float, 24> K0, CubeVals cv,
                         const uint8_t* __restrict__ bcmask, float bcdiag, const float* __restrict__ u,
                         const float* __restrict__ b, const float* __restrict__ diag, float w,
                         float* __restrict__ y, ChebArgs<float> ch, const float* __restrict__ cdiag) {
  __shared__ __align__(16) FmaSmem S;
  const int tid = threadIdx.x;
  const int nnx = g.nx + 1, nny = g.ny + 1, nnz = g.nz + 1;
  const int NX = OX + 2, EX = OX + 1;                       // staged row lengths (nodes, elements)
  const int plane = NX * (OY + 2), eplane = EX * (OY + 1);
  const int i0 = (int)blockIdx.x * OX - 1, j0 = (int)blockIdx.y * OY - 1;   // staged origin (node and element)
  const int nlay = (int)(((int64_t)nnz * (blockIdx.z + 1)) / gridDim.z) - (int)(((int64_t)nnz * blockIdx.z) / gridDim.z);
  const int kz0 = (int)(((int64_t)nnz * blockIdx.z) / gridDim.z);
  const int64_t nlayer = (int64_t)nnx * nny;
  const int64_t nn_total = nlayer * nnz;
  const int64_t elayer = (int64_t)g.nx * g.ny;
  float ca = 0.f, cc = 0.f;
  if (MODE == 3) {
    ca = (float)ch.coef[2 * ch.step];
    cc = (float)ch.coef[2 * ch.step + 1];
  }

  // staging positions of this thread (layer independent)
  int spos[FPN], gnode[FPN], epos[FPE], gelem[FPE];
#pragma unroll
  for (int s = 0; s < FPN; ++s) {
    const int v = tid + s * FT;
    const int row = v / NX, cx = v - row * NX;
    const int gi = i0 + cx, gj = j0 + row;
    spos[s] = v < plane ? v : -1;
    gnode[s] = (v < plane && gi >= 0 && gi < nnx && gj >= 0 && gj < nny) ? gj * nnx + gi : -1;
  }
#pragma unroll
  for (int s = 0; s < FPE; ++s) {
    const int v = tid + s * FT;
    const int row = v / EX, cx = v - row * EX;
    const int gi = i0 + cx, gj = j0 + row;
    epos[s] = v < eplane ? v : -1;
    gelem[s] = (v < eplane && gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny) ? gj * g.nx + gi : -1;
  }
  // the node column of this thread
  const int tx = tid % OX, ty = tid / OX;
  const int Xn = i0 + 1 + tx, Yn = j0 + 1 + ty;
  const bool owner = tid < OX * OY && Xn < nnx && Yn < nny;
  const int64_t node_xy = owner ? (int64_t)Yn * nnx + Xn : 0;
  const int wbase = ty * NX + tx;          // staged node (tx, ty): window corner
  const int ebase = ty * EX + tx;          // staged element (tx, ty)
  const int own = wbase + NX + 1;          // staged position of the owned node

  // copies of node layer kz0 - 1 + s (u, mask words) and element layer kz0 - 1 + s (x) into a slot
  auto issue = [&](int s, int slot) {
    const int ku = kz0 - 1 + s;
    const bool uok = ku >= 0 && ku < nnz, xok = ku >= 0 && ku < g.nz;
#pragma unroll
    for (int q = 0; q < FPN; ++q) {
      if (spos[q] < 0) continue;
      const bool live = uok && gnode[q] >= 0;
      const int64_t m = live ? (int64_t)ku * nlayer + gnode[q] : 0;
      const float* src = u + 3 * m;
      const int nb = live ? 4 : 0;
      float* dst = &S.u[slot][spos[q]].x;
      cp_async4(dst, src, nb);
      cp_async4(dst + 1, src + 1, nb);
      cp_async4(dst + 2, src + 2, nb);
      if (bcmask) {
        const int64_t wd = m & ~int64_t(3);
        const int64_t left = nn_total - wd;
        cp_async4(&S.m[slot][spos[q]], bcmask + wd, live ? (left < 4 ? (int)left : 4) : 0);
      }
    }
#pragma unroll
    for (int q = 0; q < FPE; ++q) {
      if (epos[q] < 0) continue;
      const bool live = xok && gelem[q] >= 0;
      cp_async4(&S.x[slot][epos[q]], xe + (live ? (int64_t)ku * elayer + gelem[q] : 0), live ? 4 : 0);
    }
    cp_async_commit();
  };
  // common shift: u at the first owned node of the tile (clamped into the grid)
  float cref[3];
  {
    const int64_t n0 = ((int64_t)min(kz0, nnz - 1) * nny + min(j0 + 1, nny - 1)) * nnx + min(i0 + 1, nnx - 1);
#pragma unroll
    for (int d = 0; d < 3; ++d) cref[d] = u[n0 * 3 + d];
  }
  // this thread's staged nodes of layer s after their copies landed: constrained dofs zeroed, shifted
  auto fixup = [&](int s, int slot) {
    const int ku = kz0 - 1 + s;
#pragma unroll
    for (int q = 0; q < FPN; ++q) {
      if (spos[q] < 0) continue;
      unsigned fixed = 0u;
      if (bcmask && gnode[q] >= 0 && ku >= 0 && ku < nnz) {
        const int64_t m = (int64_t)ku * nlayer + gnode[q];
        fixed = (S.m[slot][spos[q]] >> (8 * (int)(m & 3))) & 7u;
      }
      float4 v = S.u[slot][spos[q]];
      v.x = ((fixed & 1u) ? 0.f : v.x) - cref[0];
      v.y = ((fixed & 2u) ? 0.f : v.y) - cref[1];
      v.z = ((fixed & 4u) ? 0.f : v.z) - cref[2];
      v.w = 0.f;
      S.u[slot][spos[q]] = v;
    }
  };

  // operands of the owned node of node layer kz0 - 1 + t, loaded one layer before its output
  float ob[3] = {0.f, 0.f, 0.f}, od[3] = {1.f, 1.f, 1.f}, ou[3] = {0.f, 0.f, 0.f}, oc[3] = {0.f, 0.f, 0.f};
  float ok[3] = {0.f, 0.f, 0.f};
  auto load_operands = [&](int t) {
    if (!owner || t < 1 || t > nlay) return;
    const int64_t q0 = ((int64_t)(kz0 - 1 + t) * nlayer + node_xy) * 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (MODE >= 1) ob[d] = b[q0 + d];
      if (MODE >= 2 || cdiag) ou[d] = u[q0 + d];
      if (MODE >= 2) od[d] = diag[q0 + d];
      if (MODE == 3) oc[d] = ch.step == 0 ? 0.f : ch.d[q0 + d];
      if (cdiag) ok[d] = cdiag[q0 + d];
    }
  };

  issue(0, 0);
  issue(1, 1);
  issue(2, 2);
  load_operands(1);

  float carry[3] = {0.f, 0.f, 0.f};   // upper-face forces of the previous element layer on the owned node
  int sb = 0, st = 1, s3 = 3;         // ring slots of node layers t, t + 1 and t + 3
  for (int t = 0; t <= nlay; ++t) {
    cp_async_wait1();                 // this thread's copies of layers <= t + 1 landed
    if (t == 0) fixup(0, 0);
    fixup(t + 1, st);
    __syncthreads();
    if (t + 3 <= nlay + 1) issue(t + 3, s3);
    else cp_async_commit();           // empty group: keeps the wait counts uniform

    if (owner) {
      const int ke = kz0 - 1 + t;     // element layer between node layers t and t + 1 of the chunk
      float ab[3] = {0.f, 0.f, 0.f}, at[3] = {0.f, 0.f, 0.f};
      if (ke >= 0 && ke < g.nz) {
        float xv[4];
#pragma unroll
        for (int oy = 0; oy < 2; ++oy)
#pragma unroll
          for (int ox = 0; ox < 2; ++ox) xv[oy * 2 + ox] = S.x[sb][ebase + oy * EX + ox];
        const float4* ub = &S.u[sb][wbase];
        const float4* ut = &S.u[st][wbase];
        if (t == 0)
          element_layer<false, true, CUBE>(K0, cv, ub, ut, NX, xv, ab, at);
        else if (t == nlay)
          element_layer<true, false, CUBE>(K0, cv, ub, ut, NX, xv, ab, at);
        else
          element_layer<true, true, CUBE>(K0, cv, ub, ut, NX, xv, ab, at);
      }
      if (t >= 1) {                   // node layer kz0 - 1 + t is complete
        const int64_t n = (int64_t)(kz0 - 1 + t) * nlayer + node_xy;
        const unsigned om = bcmask ? (S.m[sb][own] >> (8 * (int)(n & 3))) & 7u : 0u;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float acc = carry[d] + ab[d];
          const int64_t q = n * 3 + d;
          const bool fixed = (om >> d) & 1u;
          float uq = ou[d];
          if (MODE < 2 && !cdiag && fixed) uq = u[q];
          float Au = fixed ? bcdiag * uq : acc;
          if (cdiag) Au += ok[d] * uq;          // constant diagonal term (AssembleStiffness add_constant)
          if (MODE == 0) {
            y[q] = Au;
          } else if (MODE == 1) {
            y[q] = ob[d] - Au;
          } else if (MODE == 2) {
            y[q] = uq + w * __fdividef(ob[d] - Au, od[d]);
          } else {
            const float dn = ca * oc[d] + cc * __fdividef(ob[d] - Au, od[d]);
            ch.d[q] = dn;
            y[q] = uq + dn;
          }
        }
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) carry[d] = at[d];
      load_operands(t + 1);
    }
    sb = st;
    st = st + 1 == FRING ? 0 : st + 1;
    s3 = s3 + 1 == FRING ? 0 : s3 + 1;
  }
  cp_async_wait_all();
}

}  // namespace

// Tile of node columns and z chunks for the grid.  Every tile width OX <= 32 that splits the x node count into
// equal parts is a candidate, with the tallest OY that fits the thread and staging limits (again split into equal
// parts); per candidate, the number of z chunks that minimises waves of CTAs x (layers per chunk + 1, the element
// layer a chunk shares with the next).  The cheapest plan wins; ties go to fewer CTAs, then to wider tiles.  At
// 128 x 64 x 64 this picks 19 x 13 columns in 8 chunks (10 layer steps per CTA) over 26 x 9 in 7 chunks (11).
static void fma_plan(const Grid& g, int slots, int& OX, int& OY, int& tx, int& ty, int& nzc) {
  const int nnx = g.nx + 1, nny = g.ny + 1, nnz = g.nz + 1;
  int64_t best = -1, best_ctas = 0;
  int best_ox = 0;
  for (int ox = 1; ox <= 32; ++ox) {
    const int cx = (nnx + ox - 1) / ox;
    if ((nnx + cx - 1) / cx != ox) continue;          // each equal-part width is visited once
    int oymax = std::min(32, FT / ox);
    while (oymax > 1 && ((ox + 2) * (oymax + 2) > FPLANE_MAX || (ox + 1) * (oymax + 1) > FEPLANE_MAX)) --oymax;
    const int cy = (nny + oymax - 1) / oymax;
    const int oy = (nny + cy - 1) / cy;
    if (cy > 65535) continue;                           // grid.y limit
    for (int c = 1; c <= nnz && c <= 65535; ++c) {      // grid.z limit
      const int64_t ctas = (int64_t)cx * cy * c;
      const int64_t cost = (ctas + slots - 1) / slots * ((nnz + c - 1) / c + 1);
      if (best < 0 || cost < best || (cost == best && (ctas < best_ctas || (ctas == best_ctas && ox > best_ox)))) {
        best = cost;
        best_ctas = ctas;
        best_ox = ox;
        OX = ox;
        OY = oy;
        tx = cx;
        ty = cy;
        nzc = c;
      }
    }
  }
}

// Class values of a cube-element K0 (true when every entry is sign x value of its class to 1e-12).
static bool cube_values(const double* K0, CubeVals& cv) {
  double val[HEX8_CLASSES];
  bool set[HEX8_CLASSES] = {};
  double amax = 0.0;
  for (int i = 0; i < 576; ++i) amax = std::max(amax, std::fabs(K0[i]));
  for (int i = 0; i < 576; ++i) {
    const int c = K0_CLASS[i];
    const double v = K0_SIGN[i] * K0[i];
    if (!set[c]) {
      val[c] = v;
      set[c] = true;
    } else if (std::fabs(v - val[c]) > 1e-12 * amax) {
      return false;
    }
  }
  for (int c = 0; c < HEX8_CLASSES; ++c) cv.v[c] = (float)val[c];
  return true;
}

template <int M, bool C>
static void launch_fma(dim3 grid, cudaStream_t st, Grid g, int OX, int OY, const float* xe,
                       const ElemMat<float, 24>& K, const CubeVals& cv, const uint8_t* bcmask, float bd,
                       const float* u, const float* b, const float* diag, float wf, float* y, ChebArgs<float> ch,
                       const float* cdiag) {
  ebe_apply_fma_kernel<M, C><<<grid, FT, 0, st>>>(g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag);
}

// 3D FP32 operator apply on the CUDA cores (modes as pmg_ebe_apply, 3 = fused Chebyshev step).
int ebe_apply_fma_f32(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                      const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                      const float* cdiag, cudaStream_t st) {
  static int resident[64][8] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch();
  if (bcmask && (reinterpret_cast<uintptr_t>(bcmask) & 3u)) {   // the mask is copied in aligned 4-byte words
    set_error("ebe_apply_fma_f32: bcmask must be 4-byte aligned");
    return PMG_BAD_ARG;
  }
  CubeVals cv = {};
  const bool cube = cube_values(K0, cv);
  const int m = mode == PMG_APPLY_MATVEC ? 0 : (mode == PMG_APPLY_RESIDUAL ? 1 : (mode == PMG_APPLY_JACOBI ? 2 : 3));
  const int key = 2 * m + (cube ? 1 : 0);
  if (!resident[dev][key]) {
    static const void* const fns[8] = {
        (const void*)ebe_apply_fma_kernel<0, false>, (const void*)ebe_apply_fma_kernel<0, true>,
        (const void*)ebe_apply_fma_kernel<1, false>, (const void*)ebe_apply_fma_kernel<1, true>,
        (const void*)ebe_apply_fma_kernel<2, false>, (const void*)ebe_apply_fma_kernel<2, true>,
        (const void*)ebe_apply_fma_kernel<3, false>, (const void*)ebe_apply_fma_kernel<3, true>};
    int r = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, fns[key], FT, 0);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      return PMG_CUDA_ERR;
    }
    resident[dev][key] = r > 0 ? r : 1;
  }
  int OX = 1, OY = 1, tx = 1, ty = 1, nzc = 1;
  fma_plan(g, resident[dev][key] * sm_count(), OX, OY, tx, ty, nzc);
  const dim3 grid(tx, ty, nzc);
  auto K = make_elem_mat<float, 24>(K0);
  const float bd = (float)bcdiag, wf = (float)w;
  switch (key) {
    case 0: launch_fma<0, false>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    case 1: launch_fma<0, true>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    case 2: launch_fma<1, false>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    case 3: launch_fma<1, true>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    case 4: launch_fma<2, false>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    case 5: launch_fma<2, true>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    case 6: launch_fma<3, false>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
    default: launch_fma<3, true>(grid, st, g, OX, OY, xe, K, cv, bcmask, bd, u, b, diag, wf, y, ch, cdiag); break;
  }
  return check_launch();
}

}  // namespace pmg

extern "C" int pmg_operator_plan(int nelx, int nely, int nelz, int slots, int* plan_host) {
  if (!pmg::grid_ok(nelx, nely, nelz) || nelz < 1 || slots < 1 || !plan_host) return PMG_BAD_ARG;
  int OX = 1, OY = 1, tx = 1, ty = 1, nzc = 1;
  pmg::fma_plan(pmg::Grid{nelx, nely, nelz}, slots, OX, OY, tx, ty, nzc);
  plan_host[0] = OX;
  plan_host[1] = OY;
  plan_host[2] = tx;
  plan_host[3] = ty;
  plan_host[4] = nzc;
  return PMG_OK;
}
