// Matrix-free hex8 operator (FP32) on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
//
// K(x) u = sum_e x_e K0 u_e (pymoto/modules/assembly.py:245-296 assembles the same sum as a CSR matrix).
//
// Work split.  A CTA (8 warps, 2 warpgroups) owns a tile of 31 x 8 elements in x, y and walks up a chunk of
// z layers.  Thread (lane l, warp r) is element (ie0 + l, je0 + r) of every layer (lane 31 is a spare whose
// scaling is zero); the CTA owns the nodes strictly inside its tile (30 x 7 per layer), so every
// contribution to an owned node is computed inside the CTA and the node sums need no atomics (deterministic
// results).  Neighbouring tiles overlap by one element in x and y.
//
// Element products without a gather.  A node layer is staged in shared memory as 16-byte records
// (ux, uy, uz, 0) in rows of exactly 32 nodes.  For the 128 elements of a warpgroup's four element rows
// (element (i, j) = A row 32 j + i), the records of their corner nodes then form the canonical K-major,
// no-swizzle operand layout: A row m at byte 16 m (SBO 128 bytes per 8 rows); the +x corner is the same
// matrix one record further (LBO 16 bytes: the second 4-column core matrix of a K = 8 slice); the +y corner
// is 32 records further; the +z corner is in the next staged layer.  So the tensor core reads A straight from
// the staged layers through shared-memory descriptors: one tcgen05.mma (M = 128, N = 32, K = 8) per corner pair
// (dy, dz) against B = K0 (K = 8 corners x 4 record entries, N = 24 forces, zero rows for the record pad).
// FP32 accuracy from three TF32 products, D = U_hi K0_hi + U_lo K0_hi + U_hi K0_lo: 12 MMAs per warpgroup and
// layer, FP32 accumulation in TMEM.  The staged displacements are taken relative to one displacement of the
// tile (K0 annihilates a common translation of an element's nodes), so the rounding error scales with the
// variation of u over the tile, not with |u|; the hi/lo split is done once per staged node.
//
// Pipeline.  Two accumulators per warpgroup: the MMAs of layer t + 1 are issued before the forces of layer t
// are read back (tcgen05.ld), scaled by x_e and summed: the upper-face forces stay in registers for the next
// layer (z), the pair of elements on either side of a node in x is summed with a warp shuffle and the pair
// in y through a small shared-memory exchange.  One CTA barrier and one mbarrier wait per layer.
//
// Staging: node layers of u, their constraint-mask words and the element layer of x are copied with cp.async
// four layers ahead into a 5-slot ring; the thread that copied a node then zeroes its constrained dofs, shifts
// it and splits it into its TF32 hi and lo records.  The operands of each thread's owned node (b, diag, u, the
// mask byte, the Chebyshev increment) are loaded into registers one layer before its output.
//
// Every wait is bounded: an mbarrier wait that gives up sets the library's operator error word
// (pmg_operator_status) and the kernel carries on to its end, where it frees its tensor memory.
#include "common.cuh"

namespace pmg {

// Error word of the tensor-core operator kernels (non-zero: a bounded wait gave up).
__device__ int g_operator_error = 0;

namespace {

constexpr int NTHREADS = 256;                // 8 warps, 2 warpgroups
constexpr uint32_t WAIT_LIMIT = 1u << 14;   // polls of at most WAIT_HINT_NS each: about a second in all
constexpr uint32_t WAIT_HINT_NS = 65536;

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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]),
        "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
      : "r"(taddr)
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
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);


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

// Tile and staging geometry.
constexpr int DX = 32, DY = 8;                  // element lanes (31 real + 1 spare) x element rows
constexpr int DNX = 32, DROWS = DY + 2;         // staged node rows of 32 records: 9 + 1 zero row read by the spare
constexpr int DPLANE = DNX * DROWS;             // 320 records
constexpr int DSTAGED = DNX * (DY + 1);         // 288 staged nodes
constexpr int DOWNX = DX - 2, DOWNY = DY - 1;   // owned nodes per tile: 30 x 7
constexpr int DRING = 5;                        // layers t .. t + 2 read by the MMAs in flight, t + 3, t + 4 copying
constexpr int DPFN = (DSTAGED + NTHREADS - 1) / NTHREADS;   // 2
constexpr int DK = 32, DN = 32;                 // GEMM K (8 corner nodes x 4) and N (24 forces + 8 zero)
constexpr int D_TMEM_COLS = 128;                // 2 warpgroups x 2 accumulators (layers t, t + 1) x 32 columns
constexpr uint32_t DB_SBO = (DK / 4) * 128;     // bytes between 8-row groups of B

struct TcSmem {
  float Bhi[DN * DK];             // [K0_hi] and [K0_lo] as K x N operands, K-major, no swizzle
  float Blo[DN * DK];
  float4 hi[DRING][DPLANE];       // staged node layers (copied, then zeroed / shifted / split in place)
  float4 lo[DRING][DPLANE];
  uint32_t m[DRING][DSTAGED];     // aligned bcmask word holding each staged node's mask byte
  float x[DRING][DX * DY];        // element layer of x (zero for the spare lane)
  float xb[2][DY][3][DX];         // y-pair exchange: [parity][row][component][lane]
  unsigned long long mbar[2][2];  // [warpgroup][accumulator]
  uint32_t tbase;
};

__device__ __forceinline__ void mma_tf32_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(IDESC), "r"(accumulate)
      : "memory");
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
  const int ie0 = (int)blockIdx.x * DOWNX - 1, je0 = (int)blockIdx.y * DOWNY - 1;
  int kz0, nlay;
  balanced_part(nnz, gridDim.z, blockIdx.z, kz0, nlay);
  const int64_t nlayer = (int64_t)nnx * nny;
  const int64_t nn_total = nlayer * nnz;
  float ca = 0.f, cc = 0.f;
  if (MODE == 3) {
    ca = (float)ch.coef[2 * ch.step];
    cc = (float)ch.coef[2 * ch.step + 1];
  }

  // B = K0 as K x N: K index 8 s + 4 xbit + c for corner pair s = (dy, dz) = (s & 1, s >> 1), x bit xbit and
  // component c (c = 3: the zero pad of the node record); N index = force row (0..23), 24..31 zero
  for (int q = tid; q < DN * DK; q += NTHREADS) {
    const int k = q / DN, n = q - (q / DN) * DN;
    const int sp = k >> 3, xbit = (k >> 2) & 1, c = k & 3;
    const int lb = xbit + 2 * (sp & 1) + 4 * (sp >> 1);
    float hi = 0.f, lo = 0.f;
    if (n < 24 && c < 3) {
      const float kv = K0.v[n * 24 + lb * 3 + c];
      hi = tf32_rna(kv);
      lo = tf32_rna(kv - hi);
    }
    const int at = (n >> 3) * (DB_SBO / 4) + (k >> 2) * 32 + (n & 7) * 4 + (k & 3);
    S.Bhi[at] = hi;
    S.Blo[at] = lo;
  }
  // the zero row read by the spare element, in every slot (never staged)
  for (int q = tid; q < DRING * (DPLANE - DSTAGED); q += NTHREADS) {
    const int sl = q / (DPLANE - DSTAGED), r = DSTAGED + q % (DPLANE - DSTAGED);
    S.hi[sl][r] = make_float4(0.f, 0.f, 0.f, 0.f);
    S.lo[sl][r] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar[q >> 1][q & 1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tbase)),
                 "r"(D_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }

  // staging slots of this thread: staged node v = row * 32 + cx (rows 0..8), node (ie0 + cx, je0 + row)
  int gnode[DPFN], spos[DPFN];
#pragma unroll
  for (int s = 0; s < DPFN; ++s) {
    const int v = tid + s * NTHREADS;
    const int row = v / DNX, cx = v - row * DNX;
    const int gi = ie0 + cx, gj = je0 + row;
    spos[s] = v < DSTAGED ? v : -1;
    gnode[s] = (v < DSTAGED && gi >= 0 && gi < nnx && gj >= 0 && gj < nny) ? gj * nnx + gi : -1;
  }
  // the element of this thread: (ie0 + lane, je0 + warp), lane 31 spare; owned node: lanes 1..30, warps 1..7
  const int Xn = ie0 + lane, Yn = je0 + warp;
  const bool owner = lane >= 1 && lane <= DX - 2 && warp >= 1 && Xn < nnx && Yn < nny;
  const int64_t node_xy = owner ? (int64_t)Yn * nnx + Xn : 0;
  const int gie = ie0 + lane, gje = je0 + warp;
  const int gelem = (lane < DX - 1 && gie >= 0 && gie < g.nx && gje >= 0 && gje < g.ny) ? gje * g.nx + gie : -1;

  auto issue = [&](int s, int slot) {
    const int ku = kz0 - 1 + s, kx = ku;
    const bool uok = ku >= 0 && ku < nnz, xok = kx >= 0 && kx < g.nz;
    const int64_t lbase = uok ? (int64_t)ku * nlayer : 0;
#pragma unroll
    for (int q = 0; q < DPFN; ++q) {
      if (spos[q] < 0) continue;
      const bool live = uok && gnode[q] >= 0;
      const int64_t m = live ? lbase + gnode[q] : 0;
      const float* src = u + 3 * m;
      const int nb = live ? 4 : 0;
      float* dst = &S.hi[slot][spos[q]].x;
      cp_async4(dst, src, nb);
      cp_async4(dst + 1, src + 1, nb);
      cp_async4(dst + 2, src + 2, nb);
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
  float cref[3];
  {
    const int64_t n0 = ((int64_t)min(kz0, nnz - 1) * nny + min(je0 + 1, nny - 1)) * nnx + min(ie0 + 1, nnx - 1);
#pragma unroll
    for (int d = 0; d < 3; ++d) cref[d] = u[n0 * 3 + d];
  }
  // this thread's staged nodes of slot s: constrained dofs zeroed, shifted by cref, split into TF32 hi (in place)
  // and lo, pad component zero
  auto fixup = [&](int s, int slot) {
    const int ku = kz0 - 1 + s;
#pragma unroll
    for (int q = 0; q < DPFN; ++q) {
      if (spos[q] < 0) continue;
      unsigned fixed = 0u;
      if (bcmask && gnode[q] >= 0 && ku >= 0 && ku < nnz) {
        const int64_t m = (int64_t)ku * nlayer + gnode[q];
        fixed = (S.m[slot][spos[q]] >> (8 * (int)(m & 3))) & 7u;
      }
      const float4 r = S.hi[slot][spos[q]];
      const float v0 = ((fixed & 1u) ? 0.f : r.x) - cref[0];
      const float v1 = ((fixed & 2u) ? 0.f : r.y) - cref[1];
      const float v2 = ((fixed & 4u) ? 0.f : r.z) - cref[2];
      const float h0 = tf32_rna(v0), h1 = tf32_rna(v1), h2 = tf32_rna(v2);
      S.hi[slot][spos[q]] = make_float4(h0, h1, h2, 0.f);
      S.lo[slot][spos[q]] = make_float4(v0 - h0, v1 - h1, v2 - h2, 0.f);
    }
  };

  const uint32_t bhi = smem_u32(S.Bhi), blo = smem_u32(S.Blo);
  const uint32_t ahi = smem_u32(S.hi), alo = smem_u32(S.lo);
  const uint32_t row0 = (uint32_t)(4 * wg) * DNX * 16u;
  // the 12 MMAs of element layer t (node layers in slots s0, s1) into accumulator buffer t & 1
  auto issue_mma = [&](int t, int s0, int s1, uint32_t tb) {
    const uint32_t sl0 = (uint32_t)s0 * DPLANE * 16u, sl1 = (uint32_t)s1 * DPLANE * 16u;
    const uint32_t dcol = tb + 64 * wg + 32 * (t & 1);
#pragma unroll
    for (int prod = 0; prod < 3; ++prod) {
      const uint32_t abase = prod == 1 ? alo : ahi;
      const uint32_t bbase = prod == 2 ? blo : bhi;
#pragma unroll
      for (int sp = 0; sp < 4; ++sp) {
        const int dy = sp & 1, dz = sp >> 1;
        const uint32_t aaddr = abase + (dz ? sl1 : sl0) + row0 + (uint32_t)dy * DNX * 16u;
        mma_tf32_ss(dcol, smem_desc(aaddr, 16u, 128u), smem_desc(bbase + 256u * sp, 128u, DB_SBO), (prod | sp) != 0);
      }
    }
    mma_commit(&S.mbar[wg][t & 1]);
  };

  // prologue: node layers 0 .. 3 copying, 0 and 1 ready, the MMAs of element layer 0 issued
  issue(0, 0);
  issue(1, 1);
  issue(2, 2);
  issue(3, 3);
  asm volatile("cp.async.wait_group 2;" ::: "memory");
  fixup(0, 0);
  fixup(1, 1);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // B, the zero rows, staged layers 0 and 1
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S.tbase;
  const uint32_t lane_sel = (uint32_t)(32 * (warp & 3)) << 16;
  if ((tid & 127) == 0) issue_mma(0, 0, 1, tbase);

  float carry[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) carry[q] = 0.f;
  float p0[3] = {0.f, 0.f, 0.f};
  float ob[3] = {0.f, 0.f, 0.f}, od[3] = {1.f, 1.f, 1.f}, ou[3] = {0.f, 0.f, 0.f}, oc[3] = {0.f, 0.f, 0.f};
  float ok[3] = {0.f, 0.f, 0.f};
  unsigned om = 0u;
  bool timed_out = false;

  // operands of the owned node of node layer kz0 - 1 + t (its mask byte included), one layer before its output
  auto load_operands = [&](int t) {
    if (!owner || t < 1 || t > nlay) return;
    const int64_t n = (int64_t)(kz0 - 1 + t) * nlayer + node_xy;
    const int64_t q0 = n * 3;
    om = bcmask ? (unsigned)bcmask[n] & 7u : 0u;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (MODE >= 1) ob[d] = b[q0 + d];
      if (MODE >= 2 || cdiag || (om >> d) & 1u) ou[d] = u[q0 + d];
      if (MODE >= 2) od[d] = diag[q0 + d];
      if (MODE == 3) oc[d] = ch.step == 0 ? 0.f : ch.d[q0 + d];
      if (cdiag) ok[d] = cdiag[q0 + d];
    }
  };
  auto node_phase = [&](int t, int xpar) {
    if (!owner || t < 1 || t > nlay) return;
    const int64_t n = (int64_t)(kz0 - 1 + t) * nlayer + node_xy;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float acc = p0[d] + S.xb[xpar][warp - 1][d][lane];
      const int64_t q = n * 3 + d;
      const bool fixed = (om >> d) & 1u;
      const float uq = ou[d];
      float Au = fixed ? bcdiag * uq : acc;
      if (cdiag) Au += ok[d] * uq;
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

  // ring slots of node layers t, t + 1, t + 2 and t + 4 (advanced without divisions)
  int sp0 = 0, sp1 = 1, sp2 = 2, sp4 = 4;
  auto next_slot = [](int v) { return v + 1 == DRING ? 0 : v + 1; };
  for (int t = 0; t <= nlay;
       ++t, sp0 = sp1, sp1 = sp2, sp2 = next_slot(sp2), sp4 = next_slot(sp4)) {
    // node layer t + 2 ready for the MMAs of element layer t + 1
    cp_async_wait1();
    fixup(t + 2, sp2);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // the slot of node layer t + 4 held layer t - 1, last read by the MMAs of element layer t - 1 (completed)
    if (t + 4 <= nlay + 1) issue(t + 4, sp4);
    else cp_async_commit();
    if ((tid & 127) == 0 && t + 1 <= nlay) issue_mma(t + 1, sp1, sp2, tbase);

    node_phase(t - 1, (t - 1) & 1);
    load_operands(t);

    // the forces of element layer t, while the tensor core runs layer t + 1
    if (!mbar_wait(&S.mbar[wg][t & 1], (uint32_t)((t >> 1) & 1))) timed_out = true;
    tc_fence_after();
    const uint32_t dcol = tbase + 64 * wg + 32 * (t & 1);
    float dv[24];
    tmem_ld16(dcol + lane_sel, dv);
    tmem_ld8(dcol + lane_sel + 16, dv + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const float xv = S.x[sp0][tid];
    float z[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      z[q] = carry[q] + xv * dv[q];
      carry[q] = xv * dv[12 + q];
    }
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
  node_phase(nlay, nlay & 1);

  cp_async_wait_all();
  if (timed_out) atomicExch(&g_operator_error, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(D_TMEM_COLS) : "memory");
  }
}

}  // namespace

// The same with the A operand read from the staged node layers (ebe_apply_tc_kernel).
int ebe_apply_tc_f32(int mode, Grid g, const float* xe, const double* K0, const uint8_t* bcmask, double bcdiag,
                      const float* u, const float* b, const float* diag, double w, float* y, ChebArgs<float> ch,
                      const float* cdiag, cudaStream_t st) {
  static bool attr_set[64][4] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch();
  if (bcmask && (reinterpret_cast<uintptr_t>(bcmask) & 3u)) {
    set_error("ebe_apply_tc_f32: bcmask must be 4-byte aligned");
    return PMG_BAD_ARG;
  }
  const size_t smem = sizeof(TcSmem) + 1024;   // two CTAs per SM: 2 x 128 TMEM columns, 2 x 77 KB
  const int m = mode == PMG_APPLY_MATVEC ? 0 : (mode == PMG_APPLY_RESIDUAL ? 1 : (mode == PMG_APPLY_JACOBI ? 2 : 3));
  const void* fn = m == 0   ? (const void*)ebe_apply_tc_kernel<0>
                   : m == 1 ? (const void*)ebe_apply_tc_kernel<1>
                   : m == 2 ? (const void*)ebe_apply_tc_kernel<2>
                            : (const void*)ebe_apply_tc_kernel<3>;
  if (!attr_set[dev][m]) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error(cudaGetErrorString(e));
      return PMG_CUDA_ERR;
    }
    attr_set[dev][m] = true;
  }
  // z chunks for two resident CTAs per SM (the occupancy query assumes the default shared-memory carveout and
  // reports one)
  const int tx = (g.nx + 1 + DOWNX - 1) / DOWNX, ty = (g.ny + 1 + DOWNY - 1) / DOWNY;
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
