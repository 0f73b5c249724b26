// Matrix-free hex8 operator (FP32) on the tensor cores.
//
// K(x) u = sum_e x_e K0 u_e (pymoto/modules/assembly.py:245-296 assembles the same sum as a CSR matrix).
// The element products F_e = K0 u_e of a whole layer of elements form one small GEMM,
// F[e][n] = sum_k U[e][k] K0[k][n] with 24 columns, issued as mma.m16n8k8 TF32 tiles.  Three TF32 products
// (hi*hi + hi*lo + lo*hi) keep FP32 accuracy, and the staged displacements are taken relative to one
// displacement of the tile (K0 annihilates rigid translations, so a common shift of all nodes of an element
// changes nothing), so the rounding error scales with the variation of u over the tile, not with |u|.
//
// A CTA owns a 32 x 8 column of nodes and walks up a chunk of z layers: per layer it stages one node layer
// of u (masked at constrained dofs) and one element layer of x in shared memory, computes the forces of the
// element layer into shared memory (no atomics), and sums the 8 element forces of every owned node of the
// layer below.  Results are deterministic.
#include "common.cuh"

namespace pmg {
namespace {

constexpr int MX = 32, MY = 8;              // maximum owned nodes per CTA in x and y
constexpr int PX = MX + 2, PY = MY + 2;     // node tile with halo (pitch of the staged u planes)
constexpr int PLANE = PX * PY;              // 340 nodes per staged layer and component
constexpr int NEMAX = (MX + 1) * (MY + 1);  // 297 elements per layer
constexpr int NMT = (NEMAX + 15) / 16;      // 19 MMA row tiles
constexpr int EPAD = 324;                   // force row pitch: >= 16*NMT and == 4 (mod 32), conflict-free stores
constexpr int NTHREADS = 256;
static_assert(MX * MY <= NTHREADS, "one owned node per thread");
constexpr int PFN = (PLANE + NTHREADS - 1) / NTHREADS;     // staged nodes per thread per layer
constexpr int PFX = (16 * NMT + NTHREADS - 1) / NTHREADS;  // staged x values per thread per layer

// Ring buffers (one barrier per layer; copies issued two layers ahead with cp.async): node layer L of u lives
// in u[(L+1)&3] and its constraint-mask words in m[(L+1)&3]; element layer L of x in x[(L+1)&3]; the forces
// of element layer L on its lower 4 nodes (rows 0..11, summed into node layer L) in lo[(L+1)&1], on its upper
// 4 nodes (rows 12..23, summed into node layer L+1) in hi[(L+1)%3].
struct MmaSmem {
  float u[4][3][PLANE];
  float x[4][16 * NMT];
  uint32_t m[4][PLANE];        // the aligned 4-byte word of bcmask holding each staged node's mask byte
  float lo[2][12][EPAD];
  float hi[3][12][EPAD];
  int etab[16 * NMT];          // element -> offset of its first node in the staged node tile
  float k0[576];
};

// 4-byte asynchronous global -> shared copy; src_bytes < 4 zero-fills the rest (0: no global read at all)
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(sa), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ uint32_t to_tf32(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Balanced split of n items into parts of at most `cap`: part p starts at `start` and has `len` items.
__device__ __forceinline__ void balanced_part(int n, int parts, int p, int& start, int& len) {
  const int base = n / parts, rem = n - base * parts;
  start = p * base + min(p, rem);
  len = base + (p < rem ? 1 : 0);
}

template <int MODE>
__global__ void __launch_bounds__(NTHREADS, 2)
    ebe_apply_mma_kernel(Grid g, const float* __restrict__ xe, ElemMat<float, 24> K0,
                         const uint8_t* __restrict__ bcmask, float bcdiag, const float* __restrict__ u,
                         const float* __restrict__ b, const float* __restrict__ diag, float w,
                         float* __restrict__ y, ChebArgs<float> ch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MmaSmem& S = *reinterpret_cast<MmaSmem*>(smem_raw);
  float* const Su = &S.u[0][0][0];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  const int nnx = g.nx + 1, nny = g.ny + 1, nnz = g.nz + 1;
  int i0, nxw, j0, nyw, kz0, nlay;
  balanced_part(nnx, gridDim.x, blockIdx.x, i0, nxw);
  balanced_part(nny, gridDim.y, blockIdx.y, j0, nyw);
  balanced_part(nnz, gridDim.z, blockIdx.z, kz0, nlay);
  const int EP = nxw + 1;                     // element tile pitch
  const int NE = EP * (nyw + 1);
  const int nmt = (NE + 15) >> 4;
  const int64_t nlayer = (int64_t)nnx * nny;
  float ca = 0.f, cc = 0.f;   // Chebyshev step coefficients (mode 3)
  if (MODE == 3) {
    ca = (float)ch.coef[2 * ch.step];
    cc = (float)ch.coef[2 * ch.step + 1];
  }

  for (int q = tid; q < 576; q += NTHREADS) S.k0[q] = K0.v[q];
  for (int e = tid; e < 16 * NMT; e += NTHREADS) {
    const int ey = e < NE ? e / EP : 0, ex = e < NE ? e - ey * EP : 0;
    S.etab[e] = ey * PX + ex;
  }
  __syncthreads();

  // B fragments of K0 (symmetric): b0 = K0[8ks+tig][8nt+gid], b1 = K0[8ks+tig+4][8nt+gid], as hi + lo TF32
  uint32_t bh[3][3][2], bl[3][3][2];
#pragma unroll
  for (int ks = 0; ks < 3; ++ks)
#pragma unroll
    for (int nt = 0; nt < 3; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float v = S.k0[(8 * ks + tig + 4 * h) * 24 + 8 * nt + gid];
        bh[ks][nt][h] = to_tf32(v);
        bl[ks][nt][h] = to_tf32(v - __uint_as_float(bh[ks][nt][h]));
      }

  // A columns of this thread: j = 2ks + h holds k = 4j + tig -> local node a = k/3, component (j + tig) % 3
  int ccol[6];
  int cz = 0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int k = 4 * j + tig, a = k / 3, d = k % 3;
    ccol[j] = d * PLANE + ((a >> 1) & 1) * PX + (a & 1);
    cz |= ((a >> 2) & 1) << j;
  }

  // staging (layer independent): node slot v of a layer -> tile position (row, cx) and node index in its layer
  int gnode[PFN], spos[PFN];
#pragma unroll
  for (int s = 0; s < PFN; ++s) {
    const int v = tid + s * NTHREADS;
    const int row = v / PX, cx = v - row * PX;
    const int gi = i0 - 1 + cx, gj = j0 - 1 + row;
    const bool inside = v < PLANE && row < nyw + 2 && cx < nxw + 2;
    spos[s] = inside ? row * PX + cx : -1;
    gnode[s] = (inside && gi >= 0 && gi < nnx && gj >= 0 && gj < nny) ? gj * nnx + gi : -1;
  }
  int gelem[PFX];
#pragma unroll
  for (int s = 0; s < PFX; ++s) {
    const int e = tid + s * NTHREADS;
    int v = -1;
    if (e < NE) {
      const int ey = e / EP, ex = e - ey * EP;
      const int gi = i0 - 1 + ex, gj = j0 - 1 + ey;
      if (gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny) v = gj * g.nx + gi;
    }
    gelem[s] = v;
  }

  // common shift of the staged displacements: u at the first owned node of the tile
  float cref[3];
  {
    const int64_t n0 = (int64_t)kz0 * nlayer + (int64_t)j0 * nnx + i0;
#pragma unroll
    for (int d = 0; d < 3; ++d) cref[d] = u[n0 * 3 + d];
  }
  const int64_t nn_total = (int64_t)nnx * nny * nnz;

  // copies of node layer L (u and its mask words) and element layer L - 1 (x), relative to kz0, one cp.async
  // group; nothing is held in registers, so the copies can be issued two layers ahead.  Slots outside the
  // grid are zero-filled without a global read.
  auto issue = [&](int L) {
    const int ku = kz0 + L, kx = kz0 + L - 1;
    const bool uok = ku >= 0 && ku < nnz, xok = kx >= 0 && kx < g.nz;
    const int ub = (L + 1) & 3;
#pragma unroll
    for (int s = 0; s < PFN; ++s) {
      if (spos[s] < 0) continue;
      const bool live = uok && gnode[s] >= 0;
      const int64_t m = live ? ku * nlayer + gnode[s] : 0;
#pragma unroll
      for (int c = 0; c < 3; ++c) cp_async4(&S.u[ub][c][spos[s]], u + m * 3 + c, live ? 4 : 0);
      if (bcmask) {
        const int64_t w = m & ~int64_t(3);    // aligned word holding the mask byte of node m
        const int64_t left = nn_total - w;
        const int bytes = live ? (left < 4 ? (int)left : 4) : 0;
        cp_async4(&S.m[ub][spos[s]], bcmask + w, bytes);
      }
    }
#pragma unroll
    for (int s = 0; s < PFX; ++s) {
      const int e = tid + s * NTHREADS;
      if (e >= 16 * NMT) continue;
      const bool live = xok && gelem[s] >= 0;
      cp_async4(&S.x[(L) & 3][e], xe + (live ? (int64_t)kx * g.nx * g.ny + gelem[s] : 0), live ? 4 : 0);
    }
    cp_async_commit();
  };
  // after this thread's copies of node layer L have landed: zero its constrained dofs and apply the shift
  // (run by the issuing thread before the barrier that publishes the layer)
  auto fixup = [&](int L) {
    const int ub = (L + 1) & 3;
    const int ku = kz0 + L;
#pragma unroll
    for (int s = 0; s < PFN; ++s) {
      if (spos[s] < 0) continue;
      unsigned keep = 7u;
      if (bcmask && gnode[s] >= 0 && ku >= 0 && ku < nnz) {
        const int64_t m = ku * nlayer + gnode[s];
        keep = ~(S.m[ub][spos[s]] >> (8 * (int)(m & 3))) & 7u;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float* p = &S.u[ub][c][spos[s]];
        *p = (((keep >> c) & 1u) ? *p : 0.f) - cref[c];
      }
    }
  };

  // element forces of one element layer: F[n][e] = x_e * sum_k u_e[k] K0[k][n]
  auto element_layer = [&](int ub0, int ub1, int xbuf, int lbuf, int hbuf) {
    int aoff[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) aoff[j] = (((cz >> j) & 1) ? ub1 : ub0) * 3 * PLANE + ccol[j];
    for (int mt = warp; mt < nmt; mt += NTHREADS / 32) {
      const int e0 = mt * 16 + gid, e1 = e0 + 8;
      const int t0 = S.etab[e0], t1 = S.etab[e1];
      float c[3][4];
#pragma unroll
      for (int nt = 0; nt < 3; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) c[nt][q] = 0.f;
#pragma unroll
      for (int ks = 0; ks < 3; ++ks) {
        uint32_t ah[4], al[4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int j = 2 * ks + h;
          const float v0 = Su[aoff[j] + t0];
          const float v1 = Su[aoff[j] + t1];
          ah[2 * h] = to_tf32(v0);                                       // a0 / a2: row gid
          al[2 * h] = __float_as_uint(v0 - __uint_as_float(ah[2 * h]));
          ah[2 * h + 1] = to_tf32(v1);                                   // a1 / a3: row gid + 8
          al[2 * h + 1] = __float_as_uint(v1 - __uint_as_float(ah[2 * h + 1]));
        }
        // consecutive MMAs go to different accumulators (dependency distance 3, not 1); small terms first
#pragma unroll
        for (int nt = 0; nt < 3; ++nt) mma_tf32(c[nt], al, bh[ks][nt][0], bh[ks][nt][1]);
#pragma unroll
        for (int nt = 0; nt < 3; ++nt) mma_tf32(c[nt], ah, bl[ks][nt][0], bl[ks][nt][1]);
#pragma unroll
        for (int nt = 0; nt < 3; ++nt) mma_tf32(c[nt], ah, bh[ks][nt][0], bh[ks][nt][1]);
      }
      const float x0 = S.x[xbuf][e0], x1 = S.x[xbuf][e1];
#pragma unroll
      for (int nt = 0; nt < 3; ++nt) {
        const int n = 8 * nt + 2 * tig;                 // rows n, n+1 lie in the same half (n even, 12 even)
        float* F = n < 12 ? &S.lo[lbuf][n][0] : &S.hi[hbuf][n - 12][0];
        F[e0] = x0 * c[nt][0];
        F[EPAD + e0] = x0 * c[nt][1];
        F[e1] = x1 * c[nt][2];
        F[EPAD + e1] = x1 * c[nt][3];
      }
    }
  };

  // Node phase operands of the owned node of this thread (MX * MY == NTHREADS: at most one), loaded before
  // the element products of the same iteration so that their latency is hidden.
  const int iy_n = tid / nxw, ix_n = tid - iy_n * nxw;
  const bool has_node = tid < nxw * nyw;
  const int64_t node_xy = (int64_t)(j0 + iy_n) * nnx + i0 + ix_n;
  float ob[3], od[3], ou[3], oc[3];
  uint8_t omask = 0;
  auto node_operands = [&](int t) {
    if (!has_node) return;
    const int64_t n = (kz0 + t) * nlayer + node_xy;
    omask = bcmask ? bcmask[n] : 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (MODE >= 1) ob[d] = b[n * 3 + d];
      if (MODE >= 2) {
        od[d] = diag[n * 3 + d];
        ou[d] = u[n * 3 + d];
      }
      if (MODE == 3) oc[d] = ch.step == 0 ? 0.f : ch.d[n * 3 + d];   // the previous step's increment
    }
  };

  // sum of the 8 element forces of the owned node of node layer L = kz0 + t
  auto node_layer = [&](int t, int lbuf, int hbuf) {
    if (!has_node) return;
    float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int e = (iy_n + oy) * EP + ix_n + ox;
        const int lxy = (1 - ox) + 2 * (1 - oy);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          acc[d] += S.lo[lbuf][3 * lxy + d][e];   // element layer L: the node is its local node lxy
          acc[d] += S.hi[hbuf][3 * lxy + d][e];   // element layer L-1: local node lxy + 4
        }
      }
    const int64_t n = (kz0 + t) * nlayer + node_xy;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int64_t q = n * 3 + d;
      const bool fixed = (omask >> d) & 1;
      if (MODE == 0) {
        y[q] = fixed ? bcdiag * u[q] : acc[d];
      } else if (MODE == 1) {
        y[q] = ob[d] - (fixed ? bcdiag * u[q] : acc[d]);
      } else if (MODE == 2) {
        const float Au = fixed ? bcdiag * ou[d] : acc[d];
        y[q] = ou[d] + w * __fdividef(ob[d] - Au, od[d]);
      } else {
        const float Au = fixed ? bcdiag * ou[d] : acc[d];
        const float dn = ca * oc[d] + cc * __fdividef(ob[d] - Au, od[d]);
        ch.d[q] = dn;
        y[q] = ou[d] + dn;
      }
    }
  };

  // prologue: node layers -1, 0 (and element layer -1) ready, node layer 1 in flight
  issue(-1);
  issue(0);
  issue(1);
  cp_async_wait1();
  fixup(-1);
  fixup(0);
  __syncthreads();
  element_layer(0, 1, 0, 0, 0);
  issue(2);

  for (int t = 0; t < nlay; ++t) {
    cp_async_wait1();                   // node layer t+1 and element layer t have landed (t+2 may be in flight)
    fixup(t + 1);
    __syncthreads();
    if (t + 3 <= nlay) issue(t + 3);
    else cp_async_commit();             // empty group: keeps the wait counts uniform
    if (t >= 1) node_operands(t - 1);
    element_layer((t + 1) & 3, (t + 2) & 3, (t + 1) & 3, (t + 1) & 1, (t + 1) % 3);
    if (t >= 1) node_layer(t - 1, t & 1, (t - 1) % 3);
  }
  node_operands(nlay - 1);
  __syncthreads();
  node_layer(nlay - 1, nlay & 1, (nlay - 1) % 3);
}

}  // namespace

// 3D FP32 operator apply on the tensor cores (modes as pmg_ebe_apply).
int ebe_apply_mma_f32(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                      const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                      cudaStream_t st) {
  static int sm_count[64] = {0};
  static bool attr_set[64][4] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch();
  if (!sm_count[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sm_count[dev] = v > 0 ? v : 1;
  }
  if (bcmask && (reinterpret_cast<uintptr_t>(bcmask) & 3u)) {   // the mask is copied in aligned 4-byte words
    set_error("ebe_apply_mma_f32: bcmask must be 4-byte aligned");
    return PMG_BAD_ARG;
  }
  const size_t smem = sizeof(MmaSmem);
  const int tx = (g.nx + 1 + MX - 1) / MX, ty = (g.ny + 1 + MY - 1) / MY;
  // z chunks: minimise (waves of two CTAs per SM) x (element layers per chunk, the halo layer included)
  const int nnz = g.nz + 1, slots = 2 * sm_count[dev];
  int nzc = 1;
  int64_t best = -1;
  for (int c = 1; c <= nnz; ++c) {
    const int64_t waves = ((int64_t)tx * ty * c + slots - 1) / slots;
    const int64_t cost = waves * ((nnz + c - 1) / c + 1);
    if (best < 0 || cost < best) {
      best = cost;
      nzc = c;
    }
  }
  const dim3 grid(tx, ty, nzc);
  auto K = make_elem_mat<float, 24>(K0);
  const int m = mode == PMG_APPLY_MATVEC ? 0 : (mode == PMG_APPLY_RESIDUAL ? 1 : (mode == PMG_APPLY_JACOBI ? 2 : 3));
  cudaError_t e = cudaSuccess;
  if (!attr_set[dev][m]) {
    const void* fn = m == 0   ? (const void*)ebe_apply_mma_kernel<0>
                     : m == 1 ? (const void*)ebe_apply_mma_kernel<1>
                     : m == 2 ? (const void*)ebe_apply_mma_kernel<2>
                              : (const void*)ebe_apply_mma_kernel<3>;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      return PMG_CUDA_ERR;
    }
    attr_set[dev][m] = true;
  }
  const float bd = (float)bcdiag, wf = (float)w;
  if (m == 0)
    ebe_apply_mma_kernel<0><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch);
  else if (m == 1)
    ebe_apply_mma_kernel<1><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch);
  else if (m == 2)
    ebe_apply_mma_kernel<2><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch);
  else
    ebe_apply_mma_kernel<3><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch);
  return check_launch();
}

}  // namespace pmg
