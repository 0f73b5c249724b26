// Kernels of the learned warm start: a small 3D convolutional network on a voxel grid (the coarse grid of
// the multigrid hierarchy), trained on the device on (density, displacement) pairs of the solver.
//
// Layout: channels-last, act[v][c] with v = (k*ny + j)*nx + i.  Activations and weights are stored as
// BF16, gradients and accumulators are FP32, master weights FP32 (Adam).  3x3x3 convolutions with zero
// padding; weights w[tap][cin][cout], tap = (dz+1)*9 + (dy+1)*3 + (dx+1).  The convolutions run on the
// tensor cores (BF16 mma.sync, FP32 accumulation).  Weight gradients are summed over fixed voxel chunks and
// then over the chunks in order, so every result is deterministic.
#include <cuda_bf16.h>

#include "common.cuh"

namespace pmg {
namespace nn {

struct VGrid {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ int64_t nvox() const { return (int64_t)nx * ny * nz; }
};

__device__ __forceinline__ void vox_ijk(const VGrid& g, int v, int& i, int& j, int& k) {
  const unsigned t = (unsigned)v / (unsigned)g.nx;
  i = v - (int)t * g.nx;
  k = (int)(t / (unsigned)g.ny);
  j = (int)t - k * g.ny;
}

__device__ __forceinline__ float ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float ld(const float* p) { return *p; }

// The three convolution products are implicit GEMMs on the tensor cores (mma.sync m16n8k16, BF16 operands,
// FP32 accumulation).  A CTA owns one 16 x 8 tile of the output; its 8 warps take interleaved 16-wide steps of
// the reduction dimension and their fragments are summed in shared memory in warp order (deterministic):
//   forward: out[v][co]  = bias[co] + sum_k A[v][k] W[k][co],  A[v][k] = in[v + off(tap)][ci],  k = tap*cin + ci
//   data:    din[v][ci]  = sum_k' D[v][k'] W'[k'][ci],  D[v][k'] = dout[v - off(tap)][co],  k' = tap*cout + co,
//                          W'[k'][ci] = w[tap][ci][co]
//   weights: dW[k][co]   = sum_v A[v][k] dout[v][co] over a chunk of voxels (the bias gradient is the extra row
//                          k = 27*cin with A = 1); chunks summed in order afterwards (deterministic).
// FP32 operands (FP32 network input, the FP32 gradients) are rounded to BF16 when the fragments are built.
constexpr int CONV_WARPS = 8;

__device__ __forceinline__ float ldf(const __nv_bfloat16* p, int64_t i) { return __bfloat162float(p[i]); }
__device__ __forceinline__ float ldf(const float* p, int64_t i) { return p[i]; }

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);     // .x (lower 16 bits) = lo
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// index of the voxel (i, j, k) + (dx, dy, dz), or -1 outside the grid
__device__ __forceinline__ int neighbour(const VGrid& g, int i, int j, int k, int dx, int dy, int dz) {
  const int ii = i + dx, jj = j + dy, kk = k + dz;
  if (ii < 0 || ii >= g.nx || jj < 0 || jj >= g.ny || kk < 0 || kk >= g.nz) return -1;
  return (kk * g.ny + jj) * g.nx + ii;
}

// A fragment of an im2col matrix: rows (voxels) r[0] = gid, r[1] = gid + 8 of the tile, columns q = tap * c + ch
// of the 16-wide step k0 (this thread's columns 2 tig + {0, 1} and 2 tig + 8 + {0, 1}); sign -1 mirrors the
// taps.  With c a multiple of 16 the step lies in one tap: one division and one neighbour per row.
template <typename T>
__device__ __forceinline__ void im2col_fragment(uint32_t (&a)[4], const VGrid& g, const T* __restrict__ x, int c,
                                                int k0, int K, const bool (&ok)[2], const int (&vi)[2],
                                                const int (&vj)[2], const int (&vk)[2], int sign, int tig) {
  if ((c & 15) == 0) {
    const int tap = k0 / c, ch0 = k0 - tap * c + 2 * tig;
    const int dx = sign * (tap % 3 - 1), dy = sign * ((tap / 3) % 3 - 1), dz = sign * (tap / 9 - 1);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int nb = ok[h] ? neighbour(g, vi[h], vj[h], vk[h], dx, dy, dz) : -1;
      const T* p = x + (int64_t)(nb < 0 ? 0 : nb) * c + ch0;
      a[h] = nb < 0 ? 0u : pack2(ldf(p, 0), ldf(p, 1));
      a[2 + h] = nb < 0 ? 0u : pack2(ldf(p, 8), ldf(p, 9));
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int h = q & 1, col = k0 + 2 * tig + 8 * (q >> 1);
    float e[2];
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int cq = col + s2;
      float v = 0.f;
      if (ok[h] && cq < K) {
        const int tap = cq / c, ch = cq - tap * c;
        const int nb = neighbour(g, vi[h], vj[h], vk[h], sign * (tap % 3 - 1), sign * ((tap / 3) % 3 - 1),
                                 sign * (tap / 9 - 1));
        if (nb >= 0) v = ldf(x, (int64_t)nb * c + ch);
      }
      e[s2] = v;
    }
    a[q] = pack2(e[0], e[1]);
  }
}

// Fragments of the CTA's warps summed in warp order; warp 0 holds the result.
__device__ __forceinline__ bool reduce_warps(float (&c)[4], float (*red)[32][4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) red[warp][lane][q] = c[q];
  __syncthreads();
  if (warp != 0) return false;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float v = red[0][lane][q];
    for (int w = 1; w < CONV_WARPS; ++w) v += red[w][lane][q];
    c[q] = v;
  }
  return true;
}

// grid (voxel tiles of 16, output-channel tiles of 8)
template <typename TIN>
__global__ void __launch_bounds__(32 * CONV_WARPS)
    conv3d_fwd_kernel(VGrid g, int cin, int cout, const TIN* __restrict__ in, const __nv_bfloat16* __restrict__ w,
                      const float* __restrict__ bias, int relu, __nv_bfloat16* __restrict__ out_bf,
                      float* __restrict__ out_f) {
  __shared__ float red[CONV_WARPS][32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gid = lane >> 2, tig = lane & 3;
  const int64_t v0 = (int64_t)blockIdx.x * 16;
  const int n = blockIdx.y * 8 + gid;
  const int64_t nv = g.nvox();
  int r[2], vi[2], vj[2], vk[2];
  bool ok[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    r[h] = (int)(v0 + gid + 8 * h);
    ok[h] = r[h] < nv;
    vox_ijk(g, ok[h] ? r[h] : 0, vi[h], vj[h], vk[h]);
  }
  const int K = 27 * cin;
  float c[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k0 = 16 * warp; k0 < K; k0 += 16 * CONV_WARPS) {
    uint32_t a[4];
    im2col_fragment(a, g, in, cin, k0, K, ok, vi, vj, vk, 1, tig);
    float bw[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int kk = k0 + 2 * tig + (q & 1) + 8 * (q >> 1);
      bw[q] = (kk < K && n < cout) ? __bfloat162float(w[(int64_t)kk * cout + n]) : 0.f;
    }
    mma_bf16(c, a, pack2(bw[0], bw[1]), pack2(bw[2], bw[3]));
  }
  if (!reduce_warps(c, red)) return;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int h = q >> 1, nc = blockIdx.y * 8 + 2 * tig + (q & 1);
    if (!ok[h] || nc >= cout) continue;
    float v = c[q] + (bias ? bias[nc] : 0.f);
    if (relu) v = fmaxf(v, 0.f);
    const int64_t o = (int64_t)r[h] * cout + nc;
    if (out_bf) out_bf[o] = __float2bfloat16(v);
    if (out_f) out_f[o] = v;
  }
}

// din[v][ci] = sum_{tap, co} w[tap][ci][co] dout[v - off(tap)][co]  (dout already masked by the ReLU);
// grid (voxel tiles of 16, input-channel tiles of 8)
__global__ void __launch_bounds__(32 * CONV_WARPS)
    conv3d_dgrad_kernel(VGrid g, int cin, int cout, const float* __restrict__ dout, const __nv_bfloat16* __restrict__ w,
                        float* __restrict__ din) {
  __shared__ float red[CONV_WARPS][32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gid = lane >> 2, tig = lane & 3;
  const int64_t v0 = (int64_t)blockIdx.x * 16;
  const int n = blockIdx.y * 8 + gid;                 // input channel
  const int64_t nv = g.nvox();
  int r[2], vi[2], vj[2], vk[2];
  bool ok[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    r[h] = (int)(v0 + gid + 8 * h);
    ok[h] = r[h] < nv;
    vox_ijk(g, ok[h] ? r[h] : 0, vi[h], vj[h], vk[h]);
  }
  const int K = 27 * cout;
  float c[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k0 = 16 * warp; k0 < K; k0 += 16 * CONV_WARPS) {
    uint32_t a[4];
    im2col_fragment(a, g, dout, cout, k0, K, ok, vi, vj, vk, -1, tig);
    float bw[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int kk = k0 + 2 * tig + (q & 1) + 8 * (q >> 1);    // tap * cout + co
      float v = 0.f;
      if (kk < K && n < cin) {
        const int tap = kk / cout, co = kk - tap * cout;
        v = __bfloat162float(w[((int64_t)tap * cin + n) * cout + co]);
      }
      bw[q] = v;
    }
    mma_bf16(c, a, pack2(bw[0], bw[1]), pack2(bw[2], bw[3]));
  }
  if (!reduce_warps(c, red)) return;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int h = q >> 1, nc = blockIdx.y * 8 + 2 * tig + (q & 1);
    if (ok[h] && nc < cin) din[(int64_t)r[h] * cin + nc] = c[q];
  }
}

// Partial weight and bias gradients over a chunk of voxels: part[chunk][k * cout + co] for k < 27 cin (k =
// tap * cin + ci) and part[chunk][27 cin cout + co] for the bias; grid (row tiles of 16, column tiles of 8,
// voxel chunks of WG_CHUNK)
constexpr int WG_CHUNK = 2048;

template <typename TIN>
__global__ void __launch_bounds__(32 * CONV_WARPS)
    conv3d_wgrad_partial_kernel(VGrid g, int cin, int cout, const TIN* __restrict__ in, const float* __restrict__ dout,
                                float* __restrict__ part) {
  __shared__ float red[CONV_WARPS][32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gid = lane >> 2, tig = lane & 3;
  const int rows = 27 * cin + 1;
  const int m0 = blockIdx.x * 16;
  const int n = blockIdx.y * 8 + gid;
  const int chunk = blockIdx.z;
  const int64_t nv = g.nvox();
  const int64_t vbeg = (int64_t)chunk * WG_CHUNK;
  const int64_t vend = min(nv, vbeg + WG_CHUNK);
  // the two rows k of this thread: tap offsets and channel (bias row: always 1; beyond: 0)
  int kind[2], ch[2], odx[2], ody[2], odz[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int kr = m0 + gid + 8 * h;
    kind[h] = kr < 27 * cin ? 0 : (kr == 27 * cin ? 1 : 2);
    const int tap = kind[h] == 0 ? kr / cin : 0;
    ch[h] = kind[h] == 0 ? kr - tap * cin : 0;
    odx[h] = tap % 3 - 1;
    ody[h] = (tap / 3) % 3 - 1;
    odz[h] = tap / 9 - 1;
  }
  float c[4] = {0.f, 0.f, 0.f, 0.f};
  for (int64_t vb = vbeg + 16 * warp; vb < vend; vb += 16 * CONV_WARPS) {
    // voxels of this thread's 4 K columns: 2tig, 2tig+1, 2tig+8, 2tig+9
    int vi[4], vj[4], vk[4];
    bool vok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t v = vb + 2 * tig + (q & 1) + 8 * (q >> 1);
      vok[q] = v < vend;
      vox_ijk(g, vok[q] ? (int)v : 0, vi[q], vj[q], vk[q]);
    }
    uint32_t a[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {          // a[q]: row gid + 8 (q & 1), columns 2tig + 8 (q >> 1) + {0, 1}
      const int h = q & 1;
      float e[2];
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int col = 2 * (q >> 1) + s2;
        float val = 0.f;
        if (vok[col]) {
          if (kind[h] == 1) {
            val = 1.f;
          } else if (kind[h] == 0) {
            const int nb = neighbour(g, vi[col], vj[col], vk[col], odx[h], ody[h], odz[h]);
            val = nb < 0 ? 0.f : ldf(in, (int64_t)nb * cin + ch[h]);
          }
        }
        e[s2] = val;
      }
      a[q] = pack2(e[0], e[1]);
    }
    float bv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t v = vb + 2 * tig + (q & 1) + 8 * (q >> 1);
      bv[q] = (v < vend && n < cout) ? dout[v * cout + n] : 0.f;
    }
    mma_bf16(c, a, pack2(bv[0], bv[1]), pack2(bv[2], bv[3]));
  }
  if (!reduce_warps(c, red)) return;
  const int nw = 27 * cin * cout + cout;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int kr = m0 + gid + 8 * (q >> 1), nc = blockIdx.y * 8 + 2 * tig + (q & 1);
    if (kr < rows && nc < cout) part[(int64_t)chunk * nw + (int64_t)kr * cout + nc] = c[q];
  }
}

__global__ void sum_chunks_kernel(int nw, int nchunk, const float* __restrict__ part, float* __restrict__ out,
                                  int accumulate) {
  const int widx = blockIdx.x * blockDim.x + threadIdx.x;
  if (widx >= nw) return;
  float acc = accumulate ? out[widx] : 0.f;
  for (int c = 0; c < nchunk; ++c) acc += part[(int64_t)c * nw + widx];
  out[widx] = acc;
}

// dout *= (act > 0)  (ReLU backward on the stored BF16 output)
__global__ void relu_bwd_kernel(int64_t n, const __nv_bfloat16* __restrict__ act, float* __restrict__ d) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n && !(__bfloat162float(act[t]) > 0.f)) d[t] = 0.f;
}

// 2x average pooling (fine grid 2nx x 2ny x 2nz -> coarse nx x ny x nz), forward and adjoint (the adjoint
// adds into its output, which also holds the gradient of the skip connection).
__global__ void pool2_fwd_kernel(VGrid gc, int c, const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= gc.nvox() * c) return;
  const int ch = (int)(t % c);
  const int v = (int)(t / c);
  int i, j, k;
  vox_ijk(gc, v, i, j, k);
  const int fx = 2 * gc.nx, fy = 2 * gc.ny;
  float acc = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int ii = 2 * i + (q & 1), jj = 2 * j + ((q >> 1) & 1), kk = 2 * k + ((q >> 2) & 1);
    acc += __bfloat162float(in[((int64_t)(kk * fy + jj) * fx + ii) * c + ch]);
  }
  out[t] = __float2bfloat16(0.125f * acc);
}

__global__ void pool2_bwd_kernel(VGrid gf, int c, const float* __restrict__ dout, float* __restrict__ din) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= gf.nvox() * c) return;
  const int ch = (int)(t % c);
  const int v = (int)(t / c);
  int i, j, k;
  vox_ijk(gf, v, i, j, k);
  const int cx = gf.nx / 2, cy = gf.ny / 2;
  din[t] += 0.125f * dout[((int64_t)((k / 2) * cy + j / 2) * cx + i / 2) * c + ch];   // accumulates
}

// 2x nearest upsampling written into channels [coff, coff+c) of a ctot-channel output (the decoder concat).
__global__ void up2_fwd_kernel(VGrid gf, int c, int ctot, int coff, const __nv_bfloat16* __restrict__ in,
                               __nv_bfloat16* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= gf.nvox() * c) return;
  const int ch = (int)(t % c);
  const int v = (int)(t / c);
  int i, j, k;
  vox_ijk(gf, v, i, j, k);
  const int cx = gf.nx / 2, cy = gf.ny / 2;
  out[(int64_t)v * ctot + coff + ch] = in[((int64_t)((k / 2) * cy + j / 2) * cx + i / 2) * c + ch];
}

// adjoint of up2: dcoarse[vc][ch] = sum over the 8 children of dfine[vf][coff + ch]
__global__ void up2_bwd_kernel(VGrid gc, int c, int ctot, int coff, const float* __restrict__ dfine,
                               float* __restrict__ dcoarse) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= gc.nvox() * c) return;
  const int ch = (int)(t % c);
  const int v = (int)(t / c);
  int i, j, k;
  vox_ijk(gc, v, i, j, k);
  const int fx = 2 * gc.nx, fy = 2 * gc.ny;
  float acc = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int ii = 2 * i + (q & 1), jj = 2 * j + ((q >> 1) & 1), kk = 2 * k + ((q >> 2) & 1);
    acc += dfine[((int64_t)(kk * fy + jj) * fx + ii) * ctot + coff + ch];
  }
  dcoarse[t] = acc;
}

// copy channels: out[v][coff + ch] = in[v][ch]  (skip connection into the concat buffer)
__global__ void copy_channels_kernel(int64_t nvox, int c, int ctot, int coff, const __nv_bfloat16* __restrict__ in,
                                     __nv_bfloat16* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nvox * c) return;
  const int ch = (int)(t % c);
  const int64_t v = t / c;
  out[v * ctot + coff + ch] = in[t];
}

// dskip[v][ch] += dcat[v][coff + ch]
__global__ void split_channels_kernel(int64_t nvox, int c, int ctot, int coff, const float* __restrict__ dcat,
                                      float* __restrict__ dskip) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nvox * c) return;
  const int ch = (int)(t % c);
  const int64_t v = t / c;
  dskip[t] += dcat[v * ctot + coff + ch];
}

// Network input on a voxel grid of stride s over the element grid: channel 0 = mean of the cube root of the
// element stiffness scaling over the s^3 elements of the voxel (a density in [0,1] under SIMP p = 3, mapped
// to 2x-1), channels 1..3 = voxel-centre coordinates in [-1,1].
__global__ void input_features_kernel(Grid ge, int s, VGrid gv, const double* __restrict__ xe,
                                      __nv_bfloat16* __restrict__ feat) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= gv.nvox()) return;
  int i, j, k;
  vox_ijk(gv, (int)v, i, j, k);
  // the feature is stored in BF16: the cube root and the mean in FP32 (no FP64 arithmetic per element)
  float acc = 0.f;
  int cnt = 0;
  const int ez = ge.nz == 0 ? 1 : ge.nz;
  for (int c = 0; c < s; ++c)
    for (int b = 0; b < s; ++b)
      for (int a = 0; a < s; ++a) {
        const int ei = i * s + a, ej = j * s + b, ek = k * s + c;
        if (ei < ge.nx && ej < ge.ny && ek < ez) {
          acc += cbrtf((float)xe[((int64_t)ek * ge.ny + ej) * ge.nx + ei]);
          ++cnt;
        }
      }
  const float m = cnt ? acc / (float)cnt : 0.f;
  feat[v * 4 + 0] = __float2bfloat16(2.f * m - 1.f);
  feat[v * 4 + 1] = __float2bfloat16(2.f * (i + 0.5f) / gv.nx - 1.f);
  feat[v * 4 + 2] = __float2bfloat16(2.f * (j + 0.5f) / gv.ny - 1.f);
  feat[v * 4 + 3] = __float2bfloat16(2.f * (k + 0.5f) / gv.nz - 1.f);
}

// Nodal field (3 components, node grid (nx+1)(ny+1)(nz+1)) from voxel values [v][3]: each node averages
// the voxels that touch it.  Adjoint: voxel gradient = sum over its 8 nodes of dnode / count(node).
__global__ void vox_to_node_kernel(VGrid gv, const float* __restrict__ vox, double* __restrict__ node) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nnx = gv.nx + 1, nny = gv.ny + 1;
  if (n >= (int64_t)nnx * nny * (gv.nz + 1)) return;
  const int i = (int)(n % nnx), j = (int)((n / nnx) % nny), k = (int)(n / ((int64_t)nnx * nny));
  float acc[3] = {0.f, 0.f, 0.f};
  int cnt = 0;
  for (int q = 0; q < 8; ++q) {
    const int vi = i - 1 + (q & 1), vj = j - 1 + ((q >> 1) & 1), vk = k - 1 + ((q >> 2) & 1);
    if (vi < 0 || vi >= gv.nx || vj < 0 || vj >= gv.ny || vk < 0 || vk >= gv.nz) continue;
    const float* p = vox + ((int64_t)(vk * gv.ny + vj) * gv.nx + vi) * 3;
    acc[0] += p[0];
    acc[1] += p[1];
    acc[2] += p[2];
    ++cnt;
  }
  const float r = cnt ? 1.f / cnt : 0.f;
  for (int d = 0; d < 3; ++d) node[n * 3 + d] = (double)(acc[d] * r);
}

__global__ void node_to_vox_adjoint_kernel(VGrid gv, const float* __restrict__ dnode, float* __restrict__ dvox) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= gv.nvox()) return;
  int i, j, k;
  vox_ijk(gv, (int)v, i, j, k);
  const int nnx = gv.nx + 1, nny = gv.ny + 1;
  float acc[3] = {0.f, 0.f, 0.f};
  for (int q = 0; q < 8; ++q) {
    const int ni = i + (q & 1), nj = j + ((q >> 1) & 1), nk = k + ((q >> 2) & 1);
    const int cx = (ni == 0 || ni == gv.nx) ? 1 : 2, cy = (nj == 0 || nj == gv.ny) ? 1 : 2,
              cz = (nk == 0 || nk == gv.nz) ? 1 : 2;
    const float r = 1.f / (cx * cy * cz);
    const float* p = dnode + ((int64_t)(nk * nny + nj) * nnx + ni) * 3;
    acc[0] += r * p[0];
    acc[1] += r * p[1];
    acc[2] += r * p[2];
  }
  for (int d = 0; d < 3; ++d) dvox[v * 3 + d] = acc[d];
}

// Adam on FP32 master weights; the BF16 copy used by the kernels is refreshed in the same pass.
__global__ void adam_kernel(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ vv, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gt = g[t] + wd * w[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * vv[t] + (1.f - b2) * gt * gt;
  m[t] = mt;
  vv[t] = vt;
  const float wn = w[t] - lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  w[t] = wn;
  if (wb) wb[t] = __float2bfloat16(wn);
}

// Weighted squared error weight * sum (pred - target)^2 on nodal values (FP64 prediction vs target) and its
// gradient (FP32); per-block partial losses (summed in block order by the caller).
__global__ void mse_kernel(int64_t n, const double* __restrict__ pred, const double* __restrict__ target,
                           double weight, float* __restrict__ grad, double* __restrict__ loss_partial) {
  __shared__ double sh[256];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (t < n) {
    const double e = pred[t] - target[t];
    l = e * e;
    grad[t] = (float)(2.0 * e * weight);
  }
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = sh[0] * weight;
}

// Injection of a nodal field of a fine grid onto the nodes of the grid coarser by `stride` (every
// stride-th node in each direction), scaled by `scale`.
__global__ void inject_kernel(Grid gf, int stride, const double* __restrict__ uf, double scale,
                              double* __restrict__ uc) {
  const int cnx = gf.nx / stride + 1, cny = gf.ny / stride + 1, cnz = gf.nz / stride + 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)cnx * cny * cnz * 3) return;
  const int d = (int)(t % 3);
  const int64_t n = t / 3;
  const int i = (int)(n % cnx), j = (int)((n / cnx) % cny), k = (int)(n / ((int64_t)cnx * cny));
  const int64_t m = ((int64_t)(k * stride) * (gf.ny + 1) + j * stride) * (gf.nx + 1) + i * stride;
  uc[t] = scale * uf[m * 3 + d];
}

}  // namespace nn
}  // namespace pmg

using namespace pmg;
using namespace pmg::nn;

static bool vgrid_ok(int nx, int ny, int nz) {
  return nx > 0 && ny > 0 && nz > 0 && (int64_t)nx * ny * nz < (int64_t(1) << 30);
}

extern "C" {

int pmg_nn_conv3d_forward(int nx, int ny, int nz, int cin, int cout, int in_is_f32, const void* in, const void* w,
                          const float* bias, int relu, void* out_bf16, float* out_f32, void* stream) {
  if (!vgrid_ok(nx, ny, nz) || cin <= 0 || cout <= 0 || !in || !w || (!out_bf16 && !out_f32)) return PMG_BAD_ARG;
  VGrid g{nx, ny, nz};
  const dim3 grid((unsigned)((g.nvox() + 15) / 16), (unsigned)((cout + 7) / 8));
  cudaStream_t st = as_stream(stream);
  const auto* wb = (const __nv_bfloat16*)w;
  auto* ob = (__nv_bfloat16*)out_bf16;
  if (in_is_f32)
    conv3d_fwd_kernel<float><<<grid, 32 * CONV_WARPS, 0, st>>>(g, cin, cout, (const float*)in, wb, bias, relu, ob,
                                                               out_f32);
  else
    conv3d_fwd_kernel<__nv_bfloat16><<<grid, 32 * CONV_WARPS, 0, st>>>(g, cin, cout, (const __nv_bfloat16*)in, wb,
                                                                       bias, relu, ob, out_f32);
  return check_launch();
}

int pmg_nn_conv3d_backward_data(int nx, int ny, int nz, int cin, int cout, const float* dout, const void* w, float* din,
                                void* stream) {
  if (!vgrid_ok(nx, ny, nz) || cin <= 0 || cout <= 0 || !dout || !w || !din) return PMG_BAD_ARG;
  VGrid g{nx, ny, nz};
  const dim3 grid((unsigned)((g.nvox() + 15) / 16), (unsigned)((cin + 7) / 8));
  conv3d_dgrad_kernel<<<grid, 32 * CONV_WARPS, 0, as_stream(stream)>>>(g, cin, cout, dout, (const __nv_bfloat16*)w,
                                                                      din);
  return check_launch();
}

size_t pmg_nn_wgrad_scratch_bytes(int nx, int ny, int nz, int cin, int cout) {
  const int64_t nv = (int64_t)nx * ny * nz;
  const int64_t nchunk = (nv + WG_CHUNK - 1) / WG_CHUNK;
  return sizeof(float) * (size_t)nchunk * (size_t)(27 * cin * cout + cout);
}

int pmg_nn_conv3d_backward_weights(int nx, int ny, int nz, int cin, int cout, int in_is_f32, const void* in,
                                   const float* dout, float* dw_db, int accumulate, void* scratch, void* stream) {
  if (!vgrid_ok(nx, ny, nz) || cin <= 0 || cout <= 0 || !in || !dout || !dw_db || !scratch) return PMG_BAD_ARG;
  VGrid g{nx, ny, nz};
  const int nw = 27 * cin * cout + cout;
  const int nchunk = (int)((g.nvox() + WG_CHUNK - 1) / WG_CHUNK);
  cudaStream_t st = as_stream(stream);
  const dim3 grid((unsigned)((27 * cin + 1 + 15) / 16), (unsigned)((cout + 7) / 8), (unsigned)nchunk);
  if (in_is_f32)
    conv3d_wgrad_partial_kernel<float><<<grid, 32 * CONV_WARPS, 0, st>>>(g, cin, cout, (const float*)in, dout,
                                                                         (float*)scratch);
  else
    conv3d_wgrad_partial_kernel<__nv_bfloat16><<<grid, 32 * CONV_WARPS, 0, st>>>(g, cin, cout,
                                                                                 (const __nv_bfloat16*)in, dout,
                                                                                 (float*)scratch);
  sum_chunks_kernel<<<(nw + 255) / 256, 256, 0, st>>>(nw, nchunk, (const float*)scratch, dw_db, accumulate);
  return check_launch();
}

int pmg_nn_relu_backward(int64_t n, const void* act_bf16, float* d, void* stream) {
  if (n < 0 || !act_bf16 || !d) return PMG_BAD_ARG;
  if (n == 0) return PMG_OK;
  relu_bwd_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(n, (const __nv_bfloat16*)act_bf16, d);
  return check_launch();
}

int pmg_nn_pool2(int direction, int cnx, int cny, int cnz, int c, const void* in, void* out, void* stream) {
  if (!vgrid_ok(cnx, cny, cnz) || c <= 0 || !in || !out) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  VGrid gc{cnx, cny, cnz};
  if (direction == 0) {
    pool2_fwd_kernel<<<blocks_for(gc.nvox() * c, 256), 256, 0, st>>>(gc, c, (const __nv_bfloat16*)in,
                                                                   (__nv_bfloat16*)out);
  } else {
    VGrid gf{2 * cnx, 2 * cny, 2 * cnz};
    pool2_bwd_kernel<<<blocks_for(gf.nvox() * c, 256), 256, 0, st>>>(gf, c, (const float*)in, (float*)out);
  }
  return check_launch();
}

int pmg_nn_up2(int direction, int cnx, int cny, int cnz, int c, int ctot, int coff, const void* in, void* out,
               void* stream) {
  if (!vgrid_ok(cnx, cny, cnz) || c <= 0 || ctot < c + coff || coff < 0 || !in || !out) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  VGrid gc{cnx, cny, cnz};
  VGrid gf{2 * cnx, 2 * cny, 2 * cnz};
  if (direction == 0)
    up2_fwd_kernel<<<blocks_for(gf.nvox() * c, 256), 256, 0, st>>>(gf, c, ctot, coff, (const __nv_bfloat16*)in,
                                                                  (__nv_bfloat16*)out);
  else
    up2_bwd_kernel<<<blocks_for(gc.nvox() * c, 256), 256, 0, st>>>(gc, c, ctot, coff, (const float*)in, (float*)out);
  return check_launch();
}

int pmg_nn_copy_channels(int64_t nvox, int c, int ctot, int coff, const void* in, void* out, void* stream) {
  if (nvox <= 0 || c <= 0 || ctot < c + coff || coff < 0 || !in || !out) return PMG_BAD_ARG;
  copy_channels_kernel<<<blocks_for(nvox * c, 256), 256, 0, as_stream(stream)>>>(nvox, c, ctot, coff,
                                                                               (const __nv_bfloat16*)in,
                                                                               (__nv_bfloat16*)out);
  return check_launch();
}

int pmg_nn_split_channels(int64_t nvox, int c, int ctot, int coff, const float* dcat, float* dskip, void* stream) {
  if (nvox <= 0 || c <= 0 || ctot < c + coff || coff < 0 || !dcat || !dskip) return PMG_BAD_ARG;
  split_channels_kernel<<<blocks_for(nvox * c, 256), 256, 0, as_stream(stream)>>>(nvox, c, ctot, coff, dcat, dskip);
  return check_launch();
}

int pmg_nn_input_features(int nelx, int nely, int nelz, int stride, int vnx, int vny, int vnz, const double* xe,
                          void* feat, void* stream) {
  if (!grid_ok(nelx, nely, nelz) || nelz == 0 || stride < 1 || !vgrid_ok(vnx, vny, vnz) || !xe || !feat)
    return PMG_BAD_ARG;
  VGrid gv{vnx, vny, vnz};
  input_features_kernel<<<blocks_for(gv.nvox(), 256), 256, 0, as_stream(stream)>>>(Grid{nelx, nely, nelz}, stride, gv,
                                                                                 xe, (__nv_bfloat16*)feat);
  return check_launch();
}

int pmg_nn_vox_to_node(int direction, int vnx, int vny, int vnz, const void* in, void* out, void* stream) {
  if (!vgrid_ok(vnx, vny, vnz) || !in || !out) return PMG_BAD_ARG;
  VGrid gv{vnx, vny, vnz};
  cudaStream_t st = as_stream(stream);
  if (direction == 0) {
    const int64_t nn = (int64_t)(vnx + 1) * (vny + 1) * (vnz + 1);
    vox_to_node_kernel<<<blocks_for(nn, 256), 256, 0, st>>>(gv, (const float*)in, (double*)out);
  } else {
    node_to_vox_adjoint_kernel<<<blocks_for(gv.nvox(), 256), 256, 0, st>>>(gv, (const float*)in, (float*)out);
  }
  return check_launch();
}

int pmg_nn_adam(int n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr, float beta1, float beta2,
                float eps, int step, float weight_decay, void* stream) {
  if (n <= 0 || !w || !g || !m || !v || step < 1) return PMG_BAD_ARG;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<(n + 255) / 256, 256, 0, as_stream(stream)>>>(n, w, g, m, v, (__nv_bfloat16*)w_bf16, lr, beta1, beta2,
                                                             eps, c1, c2, weight_decay);
  return check_launch();
}

int pmg_nn_mse(int64_t n, const double* pred, const double* target, double weight, float* grad, double* loss_partial,
               void* stream) {
  if (n <= 0 || !pred || !target || !grad || !loss_partial) return PMG_BAD_ARG;
  mse_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(n, pred, target, weight, grad, loss_partial);
  return check_launch();
}

int pmg_nn_inject(int nelx, int nely, int nelz, int stride, const double* uf, double scale, double* uc,
                  void* stream) {
  if (!grid_ok(nelx, nely, nelz) || nelz == 0 || stride < 1 || nelx % stride || nely % stride || nelz % stride ||
      !uf || !uc)
    return PMG_BAD_ARG;
  Grid gf{nelx, nely, nelz};
  const int64_t n = (int64_t)(nelx / stride + 1) * (nely / stride + 1) * (nelz / stride + 1) * 3;
  inject_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(gf, stride, uf, scale, uc);
  return check_launch();
}

}  // extern "C"
