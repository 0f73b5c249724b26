// Additive-manufacturing overhang filter (pyMOTO's OverhangFilter, pymoto/modules/filter.py:381-713), one
// launch per layer, one thread per element of the layer.
//
// Forward, layer `layer` in print order: v_k = sum over the cone window of kernel_k[m] * y_prev[e + c - m]
// (the previous layer in print order; below the first layer a baseplate of 1, beside the domain 0 -- at the
// baseplate's lateral border 1 where only axes before the print axis are outside, 0 where an axis after it is,
// as numpy's axis-by-axis padding leaves it), s = (sum_k (v_k + shift)^p)^(1/q) - backshift,
// y = (x + s - sqrt((x - s)^2 + eps) + sqrt(eps)) / 2.
// Adjoint, layers in reverse print order: an element first gathers what the later layer's supports send it
// (the transposed window: o = e - c + m), then forms dx and its own supports' derivatives
// p dsum (v_k + shift)^(p-1), written to the other half of a double buffer for the next launch.
#include "common.cuh"

namespace pmg {

struct OverhangShape {
  int n[3];      // elements per axis (nz >= 1)
  int lay, step; // print axis, +-1
  int a, b;      // the two other axes, ascending
  int w[3], c[3];
  int K;
  double p, q, shift, backshift, eps;
};

__device__ __forceinline__ int64_t oh_eid(const OverhangShape& S, const int* e3) {
  return ((int64_t)e3[2] * S.n[1] + e3[1]) * S.n[0] + e3[0];
}

// v_k of the element (ea, eb) of a layer whose support layer is `prev` (outside: the baseplate)
__device__ double oh_support(const OverhangShape& S, int k, int ea, int eb, int prev,
                             const double* __restrict__ kern, const double* __restrict__ y) {
  const bool base = prev < 0 || prev >= S.n[S.lay];
  const int wa = S.w[S.a], wb = S.w[S.b];
  const int wsz = S.w[0] * S.w[1] * S.w[2];
  double v = 0.0;
  for (int ma = 0; ma < wa; ++ma) {
    for (int mb = 0; mb < wb; ++mb) {
      int m[3] = {0, 0, 0};
      m[S.a] = ma;
      m[S.b] = mb;
      const double wk = kern[(int64_t)k * wsz + (m[0] * S.w[1] + m[1]) * S.w[2] + m[2]];
      const int ja = ea + S.c[S.a] - ma, jb = eb + S.c[S.b] - mb;
      const bool ina = ja >= 0 && ja < S.n[S.a], inb = jb >= 0 && jb < S.n[S.b];
      double val;
      if (base) {
        val = ((!ina && S.a > S.lay) || (!inb && S.b > S.lay)) ? 0.0 : 1.0;
      } else if (ina && inb) {
        int j3[3];
        j3[S.lay] = prev;
        j3[S.a] = ja;
        j3[S.b] = jb;
        val = y[oh_eid(S, j3)];
      } else {
        val = 0.0;
      }
      v += wk * val;
    }
  }
  return v;
}

__global__ void overhang_forward_kernel(OverhangShape S, int layer, const double* __restrict__ kern,
                                        const double* __restrict__ x, double* __restrict__ y,
                                        double* __restrict__ s) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int na = S.n[S.a], nb = S.n[S.b];
  if (t >= (int64_t)na * nb) return;
  const int ea = (int)(t % na), eb = (int)(t / na);
  const int prev = layer - S.step;
  double sum = 0.0;
  for (int k = 0; k < S.K; ++k) sum += pow(oh_support(S, k, ea, eb, prev, kern, y) + S.shift, S.p);
  const double sm = pow(sum, 1.0 / S.q) - S.backshift;
  int e3[3];
  e3[S.lay] = layer;
  e3[S.a] = ea;
  e3[S.b] = eb;
  const int64_t e = oh_eid(S, e3);
  const double xe = x[e], r = xe - sm;
  y[e] = (xe + sm - sqrt(r * r + S.eps) + sqrt(S.eps)) / 2;
  s[e] = sm;
}

__global__ void overhang_adjoint_kernel(OverhangShape S, int layer, int first, const double* __restrict__ kern,
                                        const double* __restrict__ x, const double* __restrict__ y,
                                        const double* __restrict__ s, const double* __restrict__ dy,
                                        double* __restrict__ dsupp_cur, const double* __restrict__ dsupp_later,
                                        double* __restrict__ dx) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int na = S.n[S.a], nb = S.n[S.b];
  const int64_t plane = (int64_t)na * nb;
  if (t >= plane) return;
  const int ea = (int)(t % na), eb = (int)(t / na);
  int e3[3];
  e3[S.lay] = layer;
  e3[S.a] = ea;
  e3[S.b] = eb;
  const int64_t e = oh_eid(S, e3);
  const int wsz = S.w[0] * S.w[1] * S.w[2];
  double d = dy[e];
  if (!first) {   // what the supports of the later layer (layer + step) send to this element
    double acc = 0.0;
    for (int ma = 0; ma < S.w[S.a]; ++ma) {
      for (int mb = 0; mb < S.w[S.b]; ++mb) {
        const int oa = ea - S.c[S.a] + ma, ob = eb - S.c[S.b] + mb;
        if (oa < 0 || oa >= na || ob < 0 || ob >= nb) continue;
        int m[3] = {0, 0, 0};
        m[S.a] = ma;
        m[S.b] = mb;
        const int mi = (m[0] * S.w[1] + m[1]) * S.w[2] + m[2];
        double part = 0.0;
        for (int k = 0; k < S.K; ++k) part += kern[(int64_t)k * wsz + mi] * dsupp_later[k * plane + oa + (int64_t)na * ob];
        acc += part;
      }
    }
    d += acc;
  }
  const double se = s[e], r = x[e] - se;
  const double dr = -d * r / (2 * sqrt(r * r + S.eps));
  dx[e] = d / 2 + dr;
  const double ds = d / 2 - dr;
  const double xsum = pow(se + S.backshift, S.q);
  const double dsum = ds * pow(xsum, 1.0 / S.q - 1.0) / S.q;
  const int prev = layer - S.step;
  if (prev < 0 || prev >= S.n[S.lay]) return;   // the first printed layer: its supports are the baseplate
  for (int k = 0; k < S.K; ++k)
    dsupp_cur[k * plane + t] = S.p * dsum * pow(oh_support(S, k, ea, eb, prev, kern, y) + S.shift, S.p - 1.0);
}

static int overhang_shape(int nx, int ny, int nz, int lay, int step, int layer, int w0, int w1, int w2, int c0,
                          int c1, int c2, int K, double p, double q, double shift, double backshift, double eps,
                          OverhangShape& S) {
  if (nx < 1 || ny < 1 || nz < 1 || lay < 0 || lay > 2 || (step != 1 && step != -1)) return PMG_BAD_ARG;
  if ((int64_t)nx * ny * nz >= ((int64_t)1 << 31) || K < 1 || K > 4096) return PMG_BAD_ARG;
  S.n[0] = nx;
  S.n[1] = ny;
  S.n[2] = nz;
  if (layer < 0 || layer >= S.n[lay]) return PMG_BAD_ARG;
  const int w[3] = {w0, w1, w2}, c[3] = {c0, c1, c2};
  S.lay = lay;
  S.step = step;
  S.a = lay == 0 ? 1 : 0;
  S.b = lay == 2 ? 1 : 2;
  for (int i = 0; i < 3; ++i) {
    if (w[i] < 1 || !(w[i] & 1) || w[i] > 255) return PMG_BAD_ARG;
    S.w[i] = w[i];
    S.c[i] = c[i];
  }
  if (w[lay] != 1 || c[lay] != step || c[S.a] != (w[S.a] - 1) / 2 || c[S.b] != (w[S.b] - 1) / 2) return PMG_BAD_ARG;
  if (!(q > 0.0) || !(eps >= 0.0)) return PMG_BAD_ARG;
  S.K = K;
  S.p = p;
  S.q = q;
  S.shift = shift;
  S.backshift = backshift;
  S.eps = eps;
  return PMG_OK;
}

}  // namespace pmg

using namespace pmg;

extern "C" {

int pmg_overhang_forward(int nx, int ny, int nz, int lay, int step, int layer, int w0, int w1, int w2, int c0, int c1,
                         int c2, int K, const double* kern, double p, double q, double shift, double backshift,
                         double eps, const double* x, double* y, double* s, void* stream) {
  OverhangShape S;
  const int rc = overhang_shape(nx, ny, nz, lay, step, layer, w0, w1, w2, c0, c1, c2, K, p, q, shift, backshift, eps,
                                S);
  if (rc != PMG_OK) return rc;
  if (!kern || !x || !y || !s || x == y || y == s) return PMG_BAD_ARG;
  const int64_t plane = (int64_t)S.n[S.a] * S.n[S.b];
  overhang_forward_kernel<<<blocks_for(plane, 128), 128, 0, as_stream(stream)>>>(S, layer, kern, x, y, s);
  return check_launch();
}

int pmg_overhang_adjoint(int nx, int ny, int nz, int lay, int step, int layer, int first, int w0, int w1, int w2,
                         int c0, int c1, int c2, int K, const double* kern, double p, double q, double shift,
                         double backshift, double eps, const double* x, const double* y, const double* s,
                         const double* dy, double* dsupp_cur, const double* dsupp_later, double* dx, void* stream) {
  OverhangShape S;
  const int rc = overhang_shape(nx, ny, nz, lay, step, layer, w0, w1, w2, c0, c1, c2, K, p, q, shift, backshift, eps,
                                S);
  if (rc != PMG_OK) return rc;
  if (!kern || !x || !y || !s || !dy || !dsupp_cur || !dx || (!first && !dsupp_later) || dsupp_cur == dsupp_later)
    return PMG_BAD_ARG;
  const int64_t plane = (int64_t)S.n[S.a] * S.n[S.b];
  overhang_adjoint_kernel<<<blocks_for(plane, 128), 128, 0, as_stream(stream)>>>(S, layer, first, kern, x, y, s, dy,
                                                                                  dsupp_cur, dsupp_later, dx);
  return check_launch();
}

}  // extern "C"
