// Matrix-free hex8 operator (FP32) on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// K(x) u = sum_e x_e K0 u_e (pymoto/modules/assembly.py:245-296 assembles the same sum as a CSR matrix).
//
// Work split.  A CTA (8 warps) owns a tile of 32 x 8 elements in x, y and walks up a chunk of z layers.
// Thread (lane l, warp r) is element (ie0 + l, je0 + r) of every layer; the CTA owns the nodes strictly
// inside its element tile (31 x 7 per layer), so every contribution to an owned node is computed inside
// the CTA and the node sums need no atomics (deterministic results).  Neighbouring tiles overlap by one
// element in x and y.
//
// Element products.  Per layer the 256 element vectors u_e (24 values) form two 128-row GEMM tiles, one
// per warpgroup: each thread writes its row into tensor memory (tcgen05.st), and one thread per
// warpgroup issues D = A B with A = [U_hi | U_lo | U_hi] (128 x 72, TF32, in TMEM) and
// B = [K0_hi; K0_hi; K0_lo] (72 x 32, TF32, in shared memory, columns 24..31 zero), so that
// D = U_hi K0_hi + U_lo K0_hi + U_hi K0_lo: three TF32 products in nine tcgen05.mma (M = 128, N = 32,
// K = 8), FP32 accumulation in TMEM.  The staged displacements are taken relative to one displacement of
// the tile (K0 annihilates a common translation of the 8 nodes of an element), so the rounding error scales
// with the variation of u over the tile, not with |u|; the hi/lo split is done once per staged node.
//
// Node sums.  The thread reads its row of D back (tcgen05.ld), scales by x_e and keeps the forces on its
// upper 4 nodes in registers for the next layer (z sum in registers); the pair of elements on either side
// of a node in x is summed with a warp shuffle, and the pair in y through a small shared-memory exchange.
// One CTA barrier, one warpgroup barrier and one mbarrier wait per layer.
//
// Staging: node layers of u, their constraint-mask words and the element layer of x are copied with cp.async
// two layers ahead into a 5-slot ring; the thread that copied a node then zeroes its constrained dofs, shifts
// it and splits it into its TF32 hi and lo parts.  The operands of each thread's owned node (b, diag, u, the
// Chebyshev increment) are loaded into registers one layer before its output.
//
// Every wait is bounded: an mbarrier wait that gives up sets the library's operator error word
// (pmg_operator_status) and the kernel carries on to its end, where it frees its tensor memory.
#include "common.cuh"

namespace pmg {

// Error word of the tensor-core operator kernels (non-zero: a bounded wait gave up).
__device__ int g_operator_error = 0;

namespace {

constexpr int TX = 32, TY = 8;               // element tile: lanes x warps
constexpr int NODX = TX + 1, NODY = TY + 1;  // staged node tile 33 x 9
constexpr int PLANE = NODX * NODY;           // 297 nodes per staged layer
constexpr int OWNX = TX - 1, OWNY = TY - 1;  // owned nodes per tile: 31 x 7
constexpr int NTHREADS = TX * TY;            // 256
constexpr int RING = 5;       // node layers t, t + 1 in use, t + 2 and t + 3 in flight, t - 1 read by the node phase
constexpr int PFN = (PLANE + NTHREADS - 1) / NTHREADS;  // staged nodes per thread: 2
constexpr int KA = 72, ND = 32;              // GEMM K (A columns) and N (D columns)
constexpr int TMEM_COLS = 256;               // 2 warpgroups x (A 72 + D 32) = 208, rounded to a power of 2
constexpr int COLS_PER_WG = KA + ND;
constexpr uint32_t WAIT_LIMIT = 1u << 14;   // polls of at most WAIT_HINT_NS each: about a second in all
constexpr uint32_t WAIT_HINT_NS = 65536;

struct TcSmem {
  float B[ND * KA];               // K-major, no swizzle: core matrix (n/8, k/4) at (n/8)*2304 + (k/4)*128 bytes
  float u[RING][3][PLANE];        // node layers of u as copied, then its TF32 hi part: [slot][component][node]
  float ulo[RING][3][PLANE];      // the lo part
  uint32_t m[RING][PLANE];        // aligned bcmask word holding each staged node's mask byte
  float x[RING][TX * TY];         // element layer of x
  float xb[2][TY][3][TX];         // y-pair exchange: [parity][row][component][lane]
  unsigned long long mbar[2];     // MMA completion, one per warpgroup
  uint32_t tbase;                 // TMEM base address from tcgen05.alloc
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(smem)), "l"(gmem), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ float tf32_rna(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
      "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]),
        "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "f"(v[0]),
               "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
               : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "r"(taddr)
               : "memory");
}

// Shared-memory matrix descriptor: no swizzle, K-major; LBO = stride between core matrices along K,
// SBO = stride between 8-row groups along M/N; bits 46-47 = 1 (descriptor version of sm_100 and later).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major, N = 32, M = 128.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t(ND) >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t B_SBO = (KA / 4) * 128;   // bytes between 8-row groups of B

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(IDESC), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(const unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Bounded wait for the mbarrier phase with the given parity; false when it gave up.
__device__ __forceinline__ bool mbar_wait(const unsigned long long* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t done;
    // the thread sleeps in the hardware until the phase completes or the hint expires: no busy polling
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(WAIT_HINT_NS)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void balanced_part(int n, int parts, int p, int& start, int& len) {
  const int base = n / parts, rem = n - base * parts;
  start = p * base + min(p, rem);
  len = base + (p < rem ? 1 : 0);
}

template <int MODE>
__global__ void __launch_bounds__(NTHREADS, 2)
    ebe_apply_tc_kernel(Grid g, const float* __restrict__ xe, ElemMat<float, 24> K0,
                        const uint8_t* __restrict__ bcmask, float bcdiag, const float* __restrict__ u,
                        const float* __restrict__ b, const float* __restrict__ diag, float w, float* __restrict__ y,
                        ChebArgs<float> ch, const float* __restrict__ cdiag) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wg = warp >> 2;
  const int nnx = g.nx + 1, nny = g.ny + 1, nnz = g.nz + 1;
  const int ie0 = (int)blockIdx.x * OWNX - 1, je0 = (int)blockIdx.y * OWNY - 1;
  int kz0, nlay;
  balanced_part(nnz, gridDim.z, blockIdx.z, kz0, nlay);
  const int64_t nlayer = (int64_t)nnx * nny;
  const int64_t nn_total = nlayer * nnz;
  float ca = 0.f, cc = 0.f;
  if (MODE == 3) {
    ca = (float)ch.coef[2 * ch.step];
    cc = (float)ch.coef[2 * ch.step + 1];
  }

  // B = [K0_hi; K0_hi; K0_lo] (72 x 32, row k, column n) in the canonical K-major layout
  for (int q = tid; q < ND * KA; q += NTHREADS) {
    const int k = q / ND, n = q - (q / ND) * ND;
    float v = 0.f;
    if (n < 24) {
      const float kv = K0.v[(k % 24) * 24 + n];
      const float hi = tf32_rna(kv);
      v = k < 48 ? hi : tf32_rna(kv - hi);
    }
    S.B[(n >> 3) * (B_SBO / 4) + (k >> 2) * 32 + (n & 7) * 4 + (k & 3)] = v;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tbase)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }

  // staging slots of this thread (layer independent): position in the staged tile and node index in its layer
  int gnode[PFN], spos[PFN];
#pragma unroll
  for (int s = 0; s < PFN; ++s) {
    const int v = tid + s * NTHREADS;
    const int row = v / NODX, cx = v - row * NODX;
    const int gi = ie0 + cx, gj = je0 + row;
    spos[s] = v < PLANE ? v : -1;
    gnode[s] = (v < PLANE && gi >= 0 && gi < nnx && gj >= 0 && gj < nny) ? gj * nnx + gi : -1;
  }
  // node owned by this thread in every layer: (ie0 + lane, je0 + warp), lane >= 1, warp >= 1
  const int Xn = ie0 + lane, Yn = je0 + warp;
  const bool owner = lane >= 1 && warp >= 1 && Xn < nnx && Yn < nny;
  const int64_t node_xy = owner ? (int64_t)Yn * nnx + Xn : 0;
  const int gie = ie0 + lane, gje = je0 + warp;
  const int gelem = (gie >= 0 && gie < g.nx && gje >= 0 && gje < g.ny) ? gje * g.nx + gie : -1;

  // copies of node layer kz0 - 1 + s (u and mask words) and element layer kz0 - 1 + s (x) into slot s % RING
  auto issue = [&](int s, int slot) {
    const int ku = kz0 - 1 + s, kx = ku;
    const bool uok = ku >= 0 && ku < nnz, xok = kx >= 0 && kx < g.nz;
    const int64_t lbase = uok ? (int64_t)ku * nlayer : 0;
#pragma unroll
    for (int q = 0; q < PFN; ++q) {
      if (spos[q] < 0) continue;
      const bool live = uok && gnode[q] >= 0;
      const int64_t m = live ? lbase + gnode[q] : 0;
      const float* src = u + 3 * m;
      const int nb = live ? 4 : 0;
      cp_async4(&S.u[slot][0][spos[q]], src, nb);
      cp_async4(&S.u[slot][1][spos[q]], src + 1, nb);
      cp_async4(&S.u[slot][2][spos[q]], src + 2, nb);
      if (bcmask) {
        const int64_t wd = m & ~int64_t(3);
        const int64_t left = nn_total - wd;
        cp_async4(&S.m[slot][spos[q]], bcmask + wd, live ? (left < 4 ? (int)left : 4) : 0);
      }
    }
    const bool xlive = xok && gelem >= 0;
    cp_async4(&S.x[slot][tid], xe + (xlive ? (int64_t)kx * g.nx * g.ny + gelem : 0), xlive ? 4 : 0);
    cp_async_commit();
  };
  // common shift of the staged displacements: u at the first owned node of the tile (clamped into the grid)
  float cref[3];
  {
    const int64_t n0 = ((int64_t)min(kz0, nnz - 1) * nny + min(je0 + 1, nny - 1)) * nnx + min(ie0 + 1, nnx - 1);
#pragma unroll
    for (int d = 0; d < 3; ++d) cref[d] = u[n0 * 3 + d];
  }
  // this thread's staged nodes of slot s (after its copies landed): constrained dofs zeroed, shifted by cref,
  // split into the TF32 hi part (in place) and the lo part
  auto fixup = [&](int s, int slot) {
    const int ku = kz0 - 1 + s;
#pragma unroll
    for (int q = 0; q < PFN; ++q) {
      if (spos[q] < 0) continue;
      unsigned fixed = 0u;
      if (bcmask && gnode[q] >= 0 && ku >= 0 && ku < nnz) {
        const int64_t m = (int64_t)ku * nlayer + gnode[q];
        fixed = (S.m[slot][spos[q]] >> (8 * (int)(m & 3))) & 7u;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float* p = &S.u[slot][c][spos[q]];
        const float v = (((fixed >> c) & 1u) ? 0.f : *p) - cref[c];
        const float hi = tf32_rna(v);
        *p = hi;
        S.ulo[slot][c][spos[q]] = v - hi;       // exact; the tensor core reads its leading TF32 bits
      }
    }
  };

  issue(0, 0);
  issue(1, 1);
  issue(2, 2);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // B and the mbarrier inits -> async proxy
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tbase;
  const uint32_t lane_sel = (uint32_t)(32 * (warp & 3)) << 16;
  const uint32_t colA = tbase + COLS_PER_WG * wg, colD = colA + KA;
  const uint32_t bbase = smem_u32(S.B);


  float carry[12];   // forces of the previous element layer on its upper nodes (local nodes 4..7)
#pragma unroll
  for (int q = 0; q < 12; ++q) carry[q] = 0.f;
  float p0[3] = {0.f, 0.f, 0.f};   // x-paired forces on node (Xn, Yn) from this element row (previous layer)
  float ob[3] = {0.f, 0.f, 0.f}, od[3] = {1.f, 1.f, 1.f}, ou[3] = {0.f, 0.f, 0.f}, oc[3] = {0.f, 0.f, 0.f};
  float ok[3] = {0.f, 0.f, 0.f};
  bool timed_out = false;

  // operands of the owned node of node layer kz0 - 1 + t, loaded into registers one layer before its output
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

  // node layer kz0 - 1 + t: the owned node's output (its mask byte was staged in slot t, its operands are in
  // registers)
  auto node_phase = [&](int t, int xpar, int slot) {
    if (!owner || t < 1 || t > nlay) return;
    const int64_t n = (int64_t)(kz0 - 1 + t) * nlayer + node_xy;
    const unsigned om = bcmask ? (S.m[slot][warp * NODX + lane] >> (8 * (int)(n & 3))) & 7u : 0u;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float acc = p0[d] + S.xb[xpar][warp - 1][d][lane];
      const int64_t q = n * 3 + d;
      const bool fixed = (om >> d) & 1u;
      float uq = ou[d];
      if (MODE < 2 && !cdiag && fixed) uq = u[q];
      float Au = fixed ? bcdiag * uq : acc;
      if (cdiag) Au += ok[d] * uq;            // constant diagonal term (AssembleStiffness add_constant)
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
  };

  // ring slots of layers t - 1, t, t + 1 and t + 3 (advanced without divisions)
  int spm1 = RING - 1, sp0 = 0, sp1 = 1, sp3 = 3;
  auto next_slot = [](int v) { return v + 1 == RING ? 0 : v + 1; };
  for (int t = 0; t <= nlay; ++t, spm1 = sp0, sp0 = sp1, sp1 = next_slot(sp1), sp3 = next_slot(sp3)) {
    // element layer kz0 - 1 + t: node layers in slots t and t + 1 (t + 1 has just landed), x in slot t
    cp_async_wait1();
    if (t == 0) fixup(0, 0);
    fixup(t + 1, sp1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t + 3 <= nlay + 1) issue(t + 3, sp3);
    else cp_async_commit();      // empty group: keeps the wait counts uniform

    // A row of this element: [u_hi | u_lo | u_hi] of its 8 nodes (staged, shifted and split)
    {
      const int s0 = sp0, s1 = sp1;
      float a[KA];
#pragma unroll
      for (int loc = 0; loc < 8; ++loc) {
        const int dx = loc & 1, dy = (loc >> 1) & 1, dz = loc >> 2;
        const int p = (warp + dy) * NODX + lane + dx;
        const int sl = dz ? s1 : s0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float hi = S.u[sl][d][p];
          a[loc * 3 + d] = hi;
          a[24 + loc * 3 + d] = S.ulo[sl][d][p];
          a[48 + loc * 3 + d] = hi;
        }
      }
      tmem_st16(colA + lane_sel, a);
      tmem_st16(colA + lane_sel + 16, a + 16);
      tmem_st16(colA + lane_sel + 32, a + 32);
      tmem_st16(colA + lane_sel + 48, a + 48);
      tmem_st8(colA + lane_sel + 64, a + 64);
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    if (wg == 0)
      asm volatile("bar.sync 1, 128;" ::: "memory");
    else
      asm volatile("bar.sync 2, 128;" ::: "memory");
    if ((tid & 127) == 0) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < KA / 8; ++s) mma_tf32(colD, colA + 8 * s, smem_desc(bbase + 256u * s, 128u, B_SBO), s > 0);
      mma_commit(&S.mbar[wg]);
    }

    // while the MMA runs: the output of node layer kz0 - 2 + t (completed in the previous iteration)
    node_phase(t - 1, (t - 1) & 1, spm1);
    load_operands(t);

    if (!mbar_wait(&S.mbar[wg], (uint32_t)(t & 1))) timed_out = true;
    tc_fence_after();
    float dv[24];
    tmem_ld16(colD + lane_sel, dv);
    tmem_ld8(colD + lane_sel + 16, dv + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const float xv = S.x[sp0][tid];
    float z[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      z[q] = carry[q] + xv * dv[q];        // local nodes 0..3: this node layer
      carry[q] = xv * dv[12 + q];          // local nodes 4..7: the next node layer
    }
    // x pairs: node (ie0 + lane, je0 + warp + ly) gets local node 2 ly of this element and local node 2 ly + 1
    // of the element to its left (lane - 1)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float l0 = __shfl_up_sync(0xffffffffu, z[3 + d], 1);
      const float l1 = __shfl_up_sync(0xffffffffu, z[9 + d], 1);
      p0[d] = z[d] + l0;
      S.xb[t & 1][warp][d][lane] = z[6 + d] + l1;
    }
    tc_fence_before();
  }
  __syncthreads();
  node_phase(nlay, nlay & 1, nlay % RING);

  cp_async_wait_all();
  if (timed_out) atomicExch(&g_operator_error, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
  }
}

}  // namespace

// 3D FP32 operator apply on the tensor cores (modes as pmg_ebe_apply, 3 = fused Chebyshev step).
int ebe_apply_tc_f32(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                     const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                     const float* cdiag, cudaStream_t st) {
  static bool attr_set[64][4] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch();
  if (bcmask && (reinterpret_cast<uintptr_t>(bcmask) & 3u)) {   // the mask is copied in aligned 4-byte words
    set_error("ebe_apply_tc_f32: bcmask must be 4-byte aligned");
    return PMG_BAD_ARG;
  }
  // at most two CTAs per SM (2 x 256 TMEM columns): the shared memory request keeps a third one out
  const size_t smem = sizeof(TcSmem) + 1024 > 80 * 1024 ? sizeof(TcSmem) + 1024 : 80 * 1024;
  const int tx = (g.nx + 1 + OWNX - 1) / OWNX, ty = (g.ny + 1 + OWNY - 1) / OWNY;
  const int nnz = g.nz + 1, slots = 2 * sm_count();
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
  if (!attr_set[dev][m]) {
    const void* fn = m == 0   ? (const void*)ebe_apply_tc_kernel<0>
                     : m == 1 ? (const void*)ebe_apply_tc_kernel<1>
                     : m == 2 ? (const void*)ebe_apply_tc_kernel<2>
                              : (const void*)ebe_apply_tc_kernel<3>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      return PMG_CUDA_ERR;
    }
    attr_set[dev][m] = true;
  }
  const float bd = (float)bcdiag, wf = (float)w;
  if (m == 0)
    ebe_apply_tc_kernel<0><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch, cdiag);
  else if (m == 1)
    ebe_apply_tc_kernel<1><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch, cdiag);
  else if (m == 2)
    ebe_apply_tc_kernel<2><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch, cdiag);
  else
    ebe_apply_tc_kernel<3><<<grid, NTHREADS, smem, st>>>(g, xe, K, bcmask, bd, u, b, diag, wf, y, ch, cdiag);
  return check_launch();
}

}  // namespace pmg

extern "C" int pmg_operator_status(int reset) {
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, pmg::g_operator_error, sizeof(int));
  if (e == cudaSuccess && reset && v) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(pmg::g_operator_error, &zero, sizeof(int));
  }
  if (e != cudaSuccess) {
    pmg::set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return v ? PMG_TIMEOUT : PMG_OK;
}
