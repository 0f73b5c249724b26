// Method of Moving Asymptotes on the device (pyMOTO's MMA.step / mmasub / subsolv,
// pymoto/common/mma.py:96-474): the asymptote adaptation, the separable approximation and the primal-dual
// interior-point Newton solution of the subproblem in ONE cooperative launch.
//
// The subproblem has n design variables and m <= PMG_MMA_MAX_M general constraints.  Its Newton iterations
// alternate O(n) element passes with O(m^2) scalar work; every element pass ends in a grid-wide reduction.
// Each CTA accumulates its elements, writes its partials and arrives at a bounded grid barrier; then EVERY CTA
// combines all partials in the same fixed order, so all CTAs hold bit-identical scalars (residual norms, the
// (m+1)x(m+1) Newton system and its solution, the step length) and take the same loop decisions without a
// second exchange.  Partials are double-buffered by barrier parity: a CTA can only overwrite a buffer after
// every CTA has passed the barrier that follows its reads.
//
// Element state (x, xsi, eta of the current iterate; the Newton direction; asymptotes, bounds, P, Q, the
// constraint gradients GG and the Newton terms delx, diagx) lives in the scratch arrays, one FP64 array each,
// read coalesced by the same thread in every pass.  A line-search trial is x_base + steg * dx evaluated on the
// fly; the accepted step is written back by the next pass that starts from the iterate.  One pass evaluates both
// the residual and the Newton system at a point, so a Newton iteration costs two passes: the direction and the
// (almost always single) line-search trial, whose pass already holds the next Newton system.
//
// Arithmetic is FP64.  The exact variant keeps the operation order of the reference, and this file is compiled
// without FMA contraction, so its element-wise values round as numpy's do; only the order of the sums over
// elements (and the (m+1)-system's elimination) differ.  The fast variant (the default of the host class)
// replaces repeated divisions by one reciprocal each; FP64 division, not memory, bounds this kernel on GB300.  Every wait is bounded (MMA_SPIN_LIMIT polls), every loop has the
// reference's iteration limits, and a singular Newton system stops the solve with a status instead of a fault.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace pmg {

constexpr int MMA_THREADS = 256;
constexpr int MMA_NW = MMA_THREADS / 32;
constexpr int MMA_MAX_BLOCKS = 1024;
constexpr int MMA_RED = 32;                     // reduction slots per pass
constexpr unsigned MMA_SPIN_LIMIT = 1u << 24;   // polls of a barrier counter before giving up
constexpr int MMA_MAX_OUTER = 400;              // epsilon levels (epsilon shrinks 10x per level)

struct MMAHeader {
  unsigned arrived[MMA_MAX_BLOCKS];
  unsigned error;   // 0 ok, 1 a barrier wait expired, 2 singular Newton system
  unsigned pad[3];
  double partial[2][MMA_MAX_BLOCKS][MMA_RED];
};

struct MMAArrays {
  int64_t n;
  const double *xval, *xold1, *xold2, *xmin, *xmax, *move, *g, *dg;
  double *offset, *low, *upp, *xnew, *info;
  double *xb, *xsib, *etab, *dxv, *dxsiv, *detav, *alfa, *beta, *rxa, *rbx, *dlx, *dgx, *P, *Q, *GG;
};

enum { RED_SUM = 0, RED_MAX = 1, RED_MIN = 2 };

// maximum / minimum that propagate NaN, as numpy's max and min do (a NaN residual then ends the Newton loop
// exactly as in the reference instead of being skipped)
__device__ __forceinline__ double nmax(double a, double b) { return (a != a || a > b) ? a : b; }
__device__ __forceinline__ double nmin(double a, double b) { return (a != a || a < b) ? a : b; }

__device__ __forceinline__ double red_op(int op, double a, double b) {
  return op == RED_SUM ? a + b : (op == RED_MAX ? nmax(a, b) : nmin(a, b));
}

__device__ __forceinline__ double warp_red(int op, double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = red_op(op, v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Arrive at barrier `gen` and wait (bounded) until every CTA has arrived.  False: abort (timeout or another
// CTA's error), uniformly for the whole CTA.
__device__ bool mma_barrier(MMAHeader* h, unsigned gen) {
  __syncthreads();
  volatile unsigned* arr = h->arrived;
  volatile unsigned* err = &h->error;
  if (threadIdx.x == 0) {
    __threadfence();
    arr[blockIdx.x] = gen;
  }
  int ok = 1;
  for (int b = threadIdx.x; ok && b < (int)gridDim.x; b += blockDim.x) {
    unsigned polls = 0;
    while (arr[b] < gen) {
      if (*err != 0u) {
        ok = 0;
        break;
      }
      if (++polls > MMA_SPIN_LIMIT) {
        atomicCAS(&h->error, 0u, 1u);
        ok = 0;
        break;
      }
    }
  }
  __threadfence();
  return __syncthreads_and(ok) != 0;
}

// Grid-wide reduction of R per-thread values: slots [0, nsum) are sums, [nsum, nsum+nmax) maxima, the rest
// minima.  Every CTA ends with the same totals in tot[].
template <int R>
__device__ bool mma_reduce(const double (&acc)[R], int nsum, int nmax, MMAHeader* h, unsigned gen, double* tot,
                           double (*wsum)[MMA_RED]) {
  static_assert(R <= MMA_RED, "too many reduction slots");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int op = r < nsum ? RED_SUM : (r < nsum + nmax ? RED_MAX : RED_MIN);
    const double v = warp_red(op, acc[r]);
    if (lane == 0) wsum[warp][r] = v;
  }
  __syncthreads();
  volatile double* part = h->partial[gen & 1u][blockIdx.x];
  if (threadIdx.x < R) {
    const int r = threadIdx.x;
    const int op = r < nsum ? RED_SUM : (r < nsum + nmax ? RED_MAX : RED_MIN);
    double v = wsum[0][r];
    for (int w = 1; w < MMA_NW; ++w) v = red_op(op, v, wsum[w][r]);
    part[r] = v;
    __threadfence();
  }
  if (!mma_barrier(h, gen)) return false;
  // the partials of all CTAs, read from L2 (the barrier's fence orders them after the arrivals), four loads in
  // flight per lane, combined in the same order in every CTA
  const int nb = (int)gridDim.x;
  for (int r = warp; r < R; r += MMA_NW) {
    const int op = r < nsum ? RED_SUM : (r < nsum + nmax ? RED_MAX : RED_MIN);
    const double* col = &h->partial[gen & 1u][0][r];
    double v = op == RED_SUM ? 0.0 : (op == RED_MAX ? -INFINITY : INFINITY);
    int b = lane;
    for (; b + 96 < nb; b += 128) {
      const double a0 = __ldcg(col + (size_t)b * MMA_RED), a1 = __ldcg(col + (size_t)(b + 32) * MMA_RED);
      const double a2 = __ldcg(col + (size_t)(b + 64) * MMA_RED), a3 = __ldcg(col + (size_t)(b + 96) * MMA_RED);
      v = red_op(op, red_op(op, red_op(op, red_op(op, v, a0), a1), a2), a3);
    }
    for (; b < nb; b += 32) v = red_op(op, v, __ldcg(col + (size_t)b * MMA_RED));
    v = warp_red(op, v);
    if (lane == 0) tot[r] = v;
  }
  __syncthreads();
  return true;
}

// acc + a * b: two roundings in the exact variant (numpy's), one fused rounding in the fast one
template <bool EXACT>
__device__ __forceinline__ double macc(double acc, double a, double b) {
  if constexpr (EXACT)
    return acc + a * b;
  else
    return fma(a, b, acc);
}

// Python's max(a, b, ...): the first of the largest (a later value replaces the current one only if greater).
__device__ __forceinline__ double py_max(const double* v, int k) {
  double r = v[0];
  for (int i = 1; i < k; ++i)
    if (v[i] > r) r = v[i];
  return r;
}

template <int M>
struct MMAScalars {
  double y[M], lam[M], mu[M], s[M], z, zet;          // current iterate
  double y0[M], lam0[M], mu0[M], s0[M], z0, zet0;    // iterate at the start of the line search
  double dy[M], dlam[M], dmu[M], ds[M], dz, dzet;    // Newton direction
  double ndy[M], ndlam[M], ndmu[M], nds[M], ndz, ndzet;   // Newton solution at the last evaluated point
  double b[M], rhs[M + 1];
  double epsi, steg, steg_used, pend, rnorm, rmax, rtry, rmaxtry;
  int has_pend, err, nbad;
};

// EXACT: every element-wise expression divides where the reference divides (values round as numpy's).
// Fast: each distinct denominator is inverted once and the quotients become products (1/(x-alfa), 1/(beta-x)
// and 1/diagx are kept from the Newton pass for the direction pass): 9 instead of 28 FP64 divisions per
// Newton iteration, each result within a few ulp of the exact one.
template <int M, bool EXACT>
__global__ void __launch_bounds__(MMA_THREADS) mma_kernel(pmg_mma_params p, MMAArrays A, MMAHeader* h) {
  constexpr int M1 = M + 1;
  __shared__ MMAScalars<M> S;
  __shared__ double tot[MMA_RED];
  __shared__ double wsum[MMA_NW][MMA_RED];
  const int64_t n = A.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t j0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned gen = 0;
  int outer = 0, newton = 0, trials = 0;

  // ---- mmasub: asymptotes, move limits, P, Q, rhs (mma.py:110-126, 176-212); subsolv's start (:282-292)
  {
    double acc[2 * M1];
#pragma unroll
    for (int r = 0; r < 2 * M1; ++r) acc[r] = 0.0;
    for (int64_t j = j0; j < n; j += stride) {
      const double xv = A.xval[j], dxr = A.xmax[j] - A.xmin[j];
      double off = A.offset[j];
      if (p.adapt) {
        const double o1 = A.xold1[j];
        const double zzz = (xv - o1) * (o1 - A.xold2[j]);
        if (zzz > 0.0)
          off = off * p.asyincr;
        else if (zzz < 0.0)
          off = off * p.asydecr;
        off = fmin(fmax(off, p.offmin), p.offmax);
        A.offset[j] = off;
      }
      const double shift = off * dxr;
      const double lo = xv - shift, up = xv + shift;
      const double al = fmax(fmax(lo + p.albefa * shift, xv - A.move[j] * dxr), A.xmin[j]);
      const double be = fmin(fmin(up - p.albefa * shift, xv + A.move[j] * dxr), A.xmax[j]);
      const double sq = shift * shift, rs = 1.0 / shift;
#pragma unroll
      for (int i = 0; i < M1; ++i) {
        const double gv = A.dg[i * n + j];
        const double dp = fmax(gv, 0.0), dm = fmax(-gv, 0.0);
        double Pv, Qv;
        if (p.version == PMG_MMA_1987) {
          Pv = sq * dp;
          Qv = sq * dm;
        } else {
          const double r = (p.version == PMG_MMA_2007 ? p.rho[0] : fmax(p.rho[i], 1e-6)) / dxr;
          Pv = sq * ((1.001 * dp + 0.001 * dm) + r);
          Qv = sq * ((0.001 * dp + 1.001 * dm) + r);
        }
        A.P[i * n + j] = Pv;
        A.Q[i * n + j] = Qv;
        acc[i] += Pv * rs;
        acc[M1 + i] += Qv * rs;
      }
      const double x = fmin(fmax(xv, al + 1e-10), be - 1e-10);
      A.xb[j] = x;
      A.xsib[j] = fmax(1.0 / (x - al), 1.0);
      A.etab[j] = fmax(1.0 / (be - x), 1.0);
      A.low[j] = lo;
      A.upp[j] = up;
      A.alfa[j] = al;
      A.beta[j] = be;
    }
    if (!mma_reduce<2 * M1>(acc, 2 * M1, 0, h, ++gen, tot, wsum)) return;
    if (threadIdx.x == 0) {
      for (int i = 0; i < M1; ++i) S.rhs[i] = (tot[i] + tot[M1 + i]) - A.g[i];
      for (int i = 0; i < M; ++i) {
        S.b[i] = S.rhs[i + 1];
        S.y[i] = 1.0;
        S.lam[i] = 1.0;
        S.mu[i] = fmax(1.0, 0.5 * p.c[i]);
        S.s[i] = 1.0;
      }
      S.z = 1.0;
      S.zet = 1.0;
      S.epsi = 1.0;
      S.has_pend = 0;
      S.pend = 0.0;
      S.err = 0;
      S.nbad = 0;
    }
    __syncthreads();
  }

  // plam = P0 + lam . P1, qlam likewise (numpy's dot(lam, P1): terms in constraint order)
  auto lam_dot = [&](const double* lam, const double* PQ, int64_t j) {
    double v = lam[0] * PQ[n + j];
#pragma unroll
    for (int i = 1; i < M; ++i) v = v + lam[i] * PQ[(i + 1) * n + j];
    return PQ[j] + v;
  };

  // Slots of the evaluation pass: [0, M) P1.(1/(upp-x)), [M, 2M) Q1.(1/(x-low)), [2M] sum of squared element
  // residuals, [2M+1, 3M+1) GG.(delx/diagx), [3M+1, 3M+1+M^2) (GG/diagx).GG^T, then the largest squared residual.
  constexpr int RS = 3 * M + 1 + M * M;
  constexpr int RE = RS + 1;

  // Newton system of dlam, dz at the evaluated point (mma.py:371-390), thread 0, from the totals in tot[].  The
  // solution goes to the n* fields: it becomes the Newton direction only if this point is kept.
  auto solve_newton = [&](double epsi) {
    double dely[M], diagy[M], AA[M1][M1], bb[M1], sol[M1];
    double alam = p.a[0] * S.lam[0];
    for (int i = 1; i < M; ++i) alam = alam + p.a[i] * S.lam[i];
    for (int i = 0; i < M; ++i) {
      const double gvec = tot[i] + tot[M + i];
      dely[i] = ((p.c[i] + p.d[i] * S.y[i]) - S.lam[i]) - epsi / S.y[i];
      const double dellam = (((gvec - p.a[i] * S.z) - S.y[i]) - S.b[i]) + epsi / S.lam[i];
      diagy[i] = p.d[i] + S.mu[i] / S.y[i];
      const double diaglamyi = S.s[i] / S.lam[i] + 1.0 / diagy[i];
      bb[i] = (dellam + dely[i] / diagy[i]) - tot[2 * M + 1 + i];
      for (int l = 0; l < M; ++l) AA[i][l] = (i == l ? diaglamyi : 0.0) + tot[3 * M + 1 + i * M + l];
      AA[i][M] = p.a[i];
      AA[M][i] = p.a[i];
    }
    AA[M][M] = -S.zet / S.z;
    bb[M] = (p.a0 - alam) - epsi / S.z;
    // LU with partial pivoting (largest magnitude in the column, first on ties), then the two triangles
    int bad = 0;
    for (int k = 0; k < M1 && !bad; ++k) {
      int pr = k;
      double amax = fabs(AA[k][k]);
      for (int i = k + 1; i < M1; ++i)
        if (fabs(AA[i][k]) > amax) {
          amax = fabs(AA[i][k]);
          pr = i;
        }
      if (!(amax > 0.0) || !isfinite(amax)) {
        bad = 1;
        break;
      }
      if (pr != k) {
        for (int c = 0; c < M1; ++c) {
          const double tmp = AA[k][c];
          AA[k][c] = AA[pr][c];
          AA[pr][c] = tmp;
        }
        const double tb = bb[k];
        bb[k] = bb[pr];
        bb[pr] = tb;
      }
      const double rinv = 1.0 / AA[k][k];
      for (int i = k + 1; i < M1; ++i) {
        const double l = AA[i][k] * rinv;
        for (int c = k + 1; c < M1; ++c) AA[i][c] = AA[i][c] - l * AA[k][c];
        bb[i] = bb[i] - l * bb[k];
      }
    }
    if (!bad) {
      for (int k = M; k >= 0; --k) {
        double v = bb[k];
        for (int c = k + 1; c < M1; ++c) v = v - AA[k][c] * sol[c];
        sol[k] = v / AA[k][k];
      }
      for (int i = 0; i < M; ++i) {
        S.ndlam[i] = sol[i];
        S.ndy[i] = -dely[i] / diagy[i] + sol[i] / diagy[i];
        S.ndmu[i] = (-S.mu[i] + epsi / S.y[i]) - (S.mu[i] * S.ndy[i]) / S.y[i];
        S.nds[i] = (-S.s[i] + epsi / S.lam[i]) - (S.s[i] * sol[i]) / S.lam[i];
      }
      S.ndz = sol[M];
      S.ndzet = (-S.zet + epsi / S.z) - (S.zet * S.ndz) / S.z;
    }
    S.nbad = bad;
  };

  // ---- one pass at a point: the KKT residual of the perturbed subproblem (mma.py:302-325) and the element terms
  // of its Newton system (mma.py:336-390).  trial: the point x_base + steg * direction of the line search;
  // otherwise the iterate, writing back a pending accepted step first.  The residual and the Newton terms share
  // 1/(upp-x), 1/(x-low), plam, qlam, dpsidx, x-alfa and beta-x, and the pass of the accepted trial already holds
  // the next Newton system, so a Newton iteration needs two passes (direction, trial) instead of three.
  auto evaluate = [&](bool trial) -> bool {
    double acc[RE];
#pragma unroll
    for (int r = 0; r < RE; ++r) acc[r] = 0.0;
    const double epsi = S.epsi;
    const bool upd = trial || S.has_pend;
    const double t = trial ? S.steg : S.pend;
    double lam[M];
#pragma unroll
    for (int i = 0; i < M; ++i) lam[i] = S.lam[i];
    for (int64_t j = j0; j < n; j += stride) {
      double x = A.xb[j], xsi = A.xsib[j], eta = A.etab[j];
      if (upd) {
        x = x + t * A.dxv[j];
        xsi = xsi + t * A.dxsiv[j];
        eta = eta + t * A.detav[j];
        if (!trial) {
          A.xb[j] = x;
          A.xsib[j] = xsi;
          A.etab[j] = eta;
        }
      }
      const double ux1 = A.upp[j] - x, xl1 = x - A.low[j];
      const double plam = lam_dot(lam, A.P, j), qlam = lam_dot(lam, A.Q, j);
      const double xa = x - A.alfa[j], bx = A.beta[j] - x;
      const double ru = 1.0 / ux1, rl = 1.0 / xl1;
      double gg[M], dpsidx, delx, diagx, rdg;
      if constexpr (EXACT) {
        const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
        const double uxinv2 = 1.0 / ux2, xlinv2 = 1.0 / xl2;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const double P1 = A.P[(i + 1) * n + j], Q1 = A.Q[(i + 1) * n + j];
          acc[i] += P1 * ru;
          acc[M + i] += Q1 * rl;
          gg[i] = P1 * uxinv2 - Q1 * xlinv2;
        }
        dpsidx = plam / ux2 - qlam / xl2;
        delx = (dpsidx - epsi / xa) + epsi / bx;
        diagx = ((2.0 * (plam / (ux1 * ux2) + qlam / (xl1 * xl2))) + xsi / xa) + eta / bx;
        rdg = 0.0;
      } else {
        const double ru2 = ru * ru, rl2 = rl * rl;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const double P1 = A.P[(i + 1) * n + j], Q1 = A.Q[(i + 1) * n + j];
          acc[i] = fma(P1, ru, acc[i]);
          acc[M + i] = fma(Q1, rl, acc[M + i]);
          gg[i] = P1 * ru2 - Q1 * rl2;
        }
        dpsidx = plam * ru2 - qlam * rl2;
        const double rxa = 1.0 / xa, rbx = 1.0 / bx;
        delx = (dpsidx - epsi * rxa) + epsi * rbx;
        diagx = ((2.0 * (plam * (ru2 * ru) + qlam * (rl2 * rl))) + xsi * rxa) + eta * rbx;
        rdg = 1.0 / diagx;
        A.rxa[j] = rxa;
        A.rbx[j] = rbx;
      }
      // residual
      const double rex = (dpsidx - xsi) + eta;
      const double rexsi = xsi * xa - epsi;
      const double reeta = eta * bx - epsi;
      const double q1 = rex * rex, q2 = rexsi * rexsi, q3 = reeta * reeta;
      acc[2 * M] += (q1 + q2) + q3;
      acc[RS] = nmax(acc[RS], nmax(nmax(q1, q2), q3));
      // Newton terms
      const double dd = EXACT ? delx / diagx : delx * rdg;
#pragma unroll
      for (int i = 0; i < M; ++i) {
        acc[2 * M + 1 + i] = macc<EXACT>(acc[2 * M + 1 + i], gg[i], dd);
        const double gi = EXACT ? gg[i] / diagx : gg[i] * rdg;
#pragma unroll
        for (int l = 0; l < M; ++l)
          acc[3 * M + 1 + i * M + l] = macc<EXACT>(acc[3 * M + 1 + i * M + l], gi, gg[l]);
      }
      A.dlx[j] = delx;
      A.dgx[j] = EXACT ? diagx : rdg;   // the fast variant keeps 1/diagx
#pragma unroll
      for (int i = 0; i < M; ++i) A.GG[i * n + j] = gg[i];
    }
    if (!mma_reduce<RE>(acc, RS, 1, h, ++gen, tot, wsum)) return false;
    if (threadIdx.x == 0) {
      double sum = tot[2 * M], mx = tot[RS];
      double alam = p.a[0] * S.lam[0];
      for (int i = 1; i < M; ++i) alam = alam + p.a[i] * S.lam[i];
      double r[4 * M + 2];
      int k = 0;
      for (int i = 0; i < M; ++i) r[k++] = ((p.c[i] + p.d[i] * S.y[i]) - S.mu[i]) - S.lam[i];
      r[k++] = (p.a0 - S.zet) - alam;
      for (int i = 0; i < M; ++i) {
        const double gvec = tot[i] + tot[M + i];
        r[k++] = (((gvec - p.a[i] * S.z) - S.y[i]) + S.s[i]) - S.b[i];
      }
      for (int i = 0; i < M; ++i) r[k++] = S.mu[i] * S.y[i] - epsi;
      r[k++] = S.zet * S.z - epsi;
      for (int i = 0; i < M; ++i) r[k++] = S.lam[i] * S.s[i] - epsi;
      for (int q = 0; q < k; ++q) {
        const double r2 = r[q] * r[q];
        sum = sum + r2;
        mx = nmax(mx, r2);
      }
      if (trial) {
        S.rtry = sum;
        S.rmaxtry = mx;
      } else {
        S.rnorm = sum;
        S.rmax = mx;
        S.has_pend = 0;
      }
      // the Newton system is needed only while the largest residual is above (0.9 epsilon)^2
      const double e9 = 0.9 * epsi;
      if (mx > e9 * e9) solve_newton(epsi);
    }
    __syncthreads();
    return true;
  };

  // ---- Newton direction of x, xsi, eta and the step length (mma.py:392-421), from the Newton system solved at
  // the kept point; writes back a pending accepted step first
  auto direction = [&]() -> bool {
    if (threadIdx.x == 0) {
      for (int i = 0; i < M; ++i) {
        S.dy[i] = S.ndy[i];
        S.dlam[i] = S.ndlam[i];
        S.dmu[i] = S.ndmu[i];
        S.ds[i] = S.nds[i];
      }
      S.dz = S.ndz;
      S.dzet = S.ndzet;
    }
    __syncthreads();
    double acc[4] = {-INFINITY, INFINITY, INFINITY, INFINITY};   // max dx/(beta-x); min dxsi/xsi, deta/eta, dx/(x-alfa)
    const double epsi = S.epsi;
    const bool upd = S.has_pend;
    const double t = S.pend;
    double dlam[M];
#pragma unroll
    for (int i = 0; i < M; ++i) dlam[i] = S.dlam[i];
    for (int64_t j = j0; j < n; j += stride) {
      double x = A.xb[j], xsi = A.xsib[j], eta = A.etab[j];
      if (upd) {
        x = x + t * A.dxv[j];
        xsi = xsi + t * A.dxsiv[j];
        eta = eta + t * A.detav[j];
        A.xb[j] = x;
        A.xsib[j] = xsi;
        A.etab[j] = eta;
      }
      const double delx = A.dlx[j];
      double dlg = dlam[0] * A.GG[j];
#pragma unroll
      for (int i = 1; i < M; ++i) dlg = dlg + dlam[i] * A.GG[i * n + j];
      double dx, dxsi, deta, rb, ra;
      if constexpr (EXACT) {
        const double diagx = A.dgx[j];
        dx = -delx / diagx - dlg / diagx;
        const double xa = x - A.alfa[j], bx = A.beta[j] - x;
        dxsi = (-xsi + epsi / xa) - (xsi * dx) / xa;
        deta = (-eta + epsi / bx) + (eta * dx) / bx;
        rb = dx / bx;
        ra = dx / xa;
      } else {
        const double rdg = A.dgx[j], rxa = A.rxa[j], rbx = A.rbx[j];
        dx = (-delx - dlg) * rdg;
        dxsi = (-xsi + epsi * rxa) - (xsi * dx) * rxa;
        deta = (-eta + epsi * rbx) + (eta * dx) * rbx;
        rb = dx * rbx;
        ra = dx * rxa;
      }
      A.dxv[j] = dx;
      A.dxsiv[j] = dxsi;
      A.detav[j] = deta;
      acc[0] = nmax(acc[0], rb);
      acc[1] = nmin(acc[1], dxsi / xsi);
      acc[2] = nmin(acc[2], deta / eta);
      acc[3] = nmin(acc[3], ra);
    }
    if (!mma_reduce<4>(acc, 0, 1, h, ++gen, tot, wsum)) return false;
    if (threadIdx.x == 0) {
      S.has_pend = 0;
      double my = S.dy[0] / S.y[0], ml = S.dlam[0] / S.lam[0], mm = S.dmu[0] / S.mu[0], ms = S.ds[0] / S.s[0];
      for (int i = 1; i < M; ++i) {
        my = nmin(my, S.dy[i] / S.y[i]);
        ml = nmin(ml, S.dlam[i] / S.lam[i]);
        mm = nmin(mm, S.dmu[i] / S.mu[i]);
        ms = nmin(ms, S.ds[i] / S.s[i]);
      }
      const double st[8] = {-1.01 * my,      -1.01 * S.dz / S.z,       -1.01 * ml, -1.01 * tot[1],
                            -1.01 * tot[2],  -1.01 * mm, -1.01 * S.dzet / S.zet, -1.01 * ms};
      const double stmxx = py_max(st, 8);
      const double last[4] = {-1.01 * tot[3], 1.01 * tot[0], stmxx, 1.0};
      S.steg = 1.0 / py_max(last, 4);
      for (int i = 0; i < M; ++i) {
        S.y0[i] = S.y[i];
        S.lam0[i] = S.lam[i];
        S.mu0[i] = S.mu[i];
        S.s0[i] = S.s[i];
      }
      S.z0 = S.z;
      S.zet0 = S.zet;
    }
    __syncthreads();
    return true;
  };

  // ---- subsolv's epsilon loop (mma.py:295-472)
  for (;;) {
    const bool more = S.epsi > p.epsimin && outer < MMA_MAX_OUTER;
    __syncthreads();
    if (!more) break;
    ++outer;
    if (!evaluate(false)) return;
    for (int it = 0; it < p.maxit; ++it) {
      const double e9 = 0.9 * S.epsi;
      const bool go = S.rmax > e9 * e9;
      const int bad = S.nbad;
      __syncthreads();
      if (!go) break;
      ++newton;
      if (bad) {   // the reference's linear solve would raise here
        if (threadIdx.x == 0) atomicCAS(&h->error, 0u, 2u);
        return;
      }
      if (!direction()) return;
      // line search: halve the step until the residual norm decreases (mma.py:436-468)
      for (int ls = 0; ls < p.maxit; ++ls) {
        ++trials;
        if (threadIdx.x == 0) {
          const double st = S.steg;
          for (int i = 0; i < M; ++i) {
            S.y[i] = S.y0[i] + st * S.dy[i];
            S.lam[i] = S.lam0[i] + st * S.dlam[i];
            S.mu[i] = S.mu0[i] + st * S.dmu[i];
            S.s[i] = S.s0[i] + st * S.ds[i];
          }
          S.z = S.z0 + st * S.dz;
          S.zet = S.zet0 + st * S.dzet;
          S.steg_used = st;
        }
        __syncthreads();
        if (!evaluate(true)) return;
        const bool accept = S.rtry < S.rnorm;
        __syncthreads();
        if (accept) break;
        if (threadIdx.x == 0) S.steg = S.steg / 2;
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        S.rnorm = S.rtry;
        S.rmax = S.rmaxtry;
        S.pend = S.steg_used;
        S.has_pend = 1;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) S.epsi = S.epsi / 10;
    __syncthreads();
  }

  // ---- the new design, gest and dk (mma.py:222-232)
  {
    double acc[M1 + 1];
#pragma unroll
    for (int r = 0; r < M1 + 1; ++r) acc[r] = 0.0;
    const bool upd = S.has_pend;
    const double t = S.pend;
    for (int64_t j = j0; j < n; j += stride) {
      double x = A.xb[j];
      if (upd) x = x + t * A.dxv[j];
      A.xnew[j] = x;
      const double lo = A.low[j], up = A.upp[j];
      const double ux = up - x, xl = x - lo;
#pragma unroll
      for (int i = 0; i < M1; ++i) acc[i] += A.P[i * n + j] / ux + A.Q[i * n + j] / xl;
      const double d = x - A.xval[j], dxr = A.xmax[j] - A.xmin[j];
      acc[M1] += ((up - lo) * (d * d)) / ((ux * xl) * dxr);
    }
    if (!mma_reduce<M1 + 1>(acc, M1 + 1, 0, h, ++gen, tot, wsum)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      for (int i = 0; i < M1; ++i) A.info[i] = tot[i] - S.rhs[i];
      A.info[M1] = tot[M1];
      A.info[M1 + 2] = (double)outer;
      A.info[M1 + 3] = (double)newton;
      A.info[M1 + 4] = (double)trials;
    }
  }
}

__global__ void mma_init_kernel(MMAHeader* h) {
  for (int b = threadIdx.x; b < MMA_MAX_BLOCKS; b += blockDim.x) h->arrived[b] = 0u;
  if (threadIdx.x == 0) h->error = 0u;
}

__global__ void mma_status_kernel(const MMAHeader* h, double* info, int m) {
  if (threadIdx.x == 0) info[m + 2] = (double)h->error;
}

inline size_t mma_header_bytes() { return (sizeof(MMAHeader) + 255) & ~size_t(255); }

template <int M, bool EXACT>
int mma_launch(const pmg_mma_params& p, const MMAArrays& A, MMAHeader* h, cudaStream_t st) {
  static int max_blocks[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    set_error("no current CUDA device");
    return PMG_CUDA_ERR;
  }
  if (max_blocks[dev] == 0) {
    int sms = 0, per_sm = 0, coop = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mma_kernel<M, EXACT>, MMA_THREADS, 0);
    max_blocks[dev] = coop && per_sm > 0 ? std::min(sms * per_sm, MMA_MAX_BLOCKS) : -1;
  }
  if (max_blocks[dev] < 0) {
    set_error("the MMA update needs a cooperative launch, which this device does not support");
    return PMG_CUDA_ERR;
  }
  const int64_t want = (A.n + MMA_THREADS - 1) / MMA_THREADS;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, max_blocks[dev]));
  pmg_mma_params pc = p;
  MMAArrays Ac = A;
  void* args[] = {(void*)&pc, (void*)&Ac, (void*)&h};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)mma_kernel<M, EXACT>, dim3(grid), dim3(MMA_THREADS), args, 0, st);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return PMG_CUDA_ERR;
  }
  return PMG_OK;
}

}  // namespace pmg

using namespace pmg;

extern "C" {

size_t pmg_mma_scratch_bytes(int64_t n, int m) {
  if (n <= 0 || m < 1 || m > PMG_MMA_MAX_M) return 0;
  return mma_header_bytes() + (size_t)(12 + 2 * (m + 1) + m) * (size_t)n * sizeof(double);
}

int pmg_mma_update(int64_t n, const pmg_mma_params* params_host, const double* xval, const double* xold1,
                   const double* xold2, const double* xmin, const double* xmax, const double* move, const double* g,
                   const double* dg, double* offset, double* low, double* upp, double* xnew, double* info,
                   void* scratch, void* stream) {
  if (n <= 0 || !params_host || !xval || !xmin || !xmax || !move || !g || !dg || !offset || !low || !upp || !xnew ||
      !info || !scratch)
    return PMG_BAD_ARG;
  const pmg_mma_params& p = *params_host;
  if (p.m < 1 || p.m > PMG_MMA_MAX_M || p.maxit < 1 || p.maxit > 100000 || !(p.epsimin > 0.0)) return PMG_BAD_ARG;
  if (p.exact != 0 && p.exact != 1) return PMG_BAD_ARG;
  if (p.version != PMG_MMA_1987 && p.version != PMG_MMA_2007 && p.version != PMG_MMA_GCMMA) return PMG_BAD_ARG;
  if (p.adapt && (!xold1 || !xold2)) return PMG_BAD_ARG;
  if (xnew == xval || xnew == low || xnew == upp || low == upp || offset == xnew) return PMG_BAD_ARG;
  if (n > (int64_t)1 << 40) return PMG_BAD_ARG;
  cudaStream_t st = as_stream(stream);
  MMAHeader* h = (MMAHeader*)scratch;
  double* arr = (double*)((char*)scratch + mma_header_bytes());
  MMAArrays A;
  A.n = n;
  A.xval = xval;
  A.xold1 = xold1;
  A.xold2 = xold2;
  A.xmin = xmin;
  A.xmax = xmax;
  A.move = move;
  A.g = g;
  A.dg = dg;
  A.offset = offset;
  A.low = low;
  A.upp = upp;
  A.xnew = xnew;
  A.info = info;
  double** slots[] = {&A.xb, &A.xsib, &A.etab, &A.dxv, &A.dxsiv, &A.detav, &A.alfa, &A.beta, &A.rxa, &A.rbx,
                      &A.dlx, &A.dgx};
  for (double** s : slots) {
    *s = arr;
    arr += n;
  }
  A.P = arr;
  arr += (p.m + 1) * n;
  A.Q = arr;
  arr += (p.m + 1) * n;
  A.GG = arr;
  mma_init_kernel<<<1, 256, 0, st>>>(h);
  int rc;
  if (p.exact) {
    switch (p.m) {
      case 1: rc = mma_launch<1, true>(p, A, h, st); break;
      case 2: rc = mma_launch<2, true>(p, A, h, st); break;
      case 3: rc = mma_launch<3, true>(p, A, h, st); break;
      default: rc = mma_launch<4, true>(p, A, h, st); break;
    }
  } else {
    switch (p.m) {
      case 1: rc = mma_launch<1, false>(p, A, h, st); break;
      case 2: rc = mma_launch<2, false>(p, A, h, st); break;
      case 3: rc = mma_launch<3, false>(p, A, h, st); break;
      default: rc = mma_launch<4, false>(p, A, h, st); break;
    }
  }
  if (rc != PMG_OK) return rc;
  mma_status_kernel<<<1, 32, 0, st>>>(h, info, p.m);
  return check_launch();
}

}  // extern "C"
