// Library identification and error reporting of the C ABI.
#include <cmath>

#include "common.cuh"

namespace pmg {
static thread_local char g_last_error[256] = "";

void set_error(const char* msg) {
  std::strncpy(g_last_error, msg ? msg : "", sizeof(g_last_error) - 1);
  g_last_error[sizeof(g_last_error) - 1] = '\0';
}

const char* last_error() { return g_last_error; }
}  // namespace pmg

extern "C" {

int pmg_version(void) { return 100; }

const char* pmg_status_string(int status) {
  switch (status) {
    case PMG_OK: return "ok";
    case PMG_BAD_ARG: return "invalid argument";
    case PMG_NOT_CONVERGED: return "not converged";
    case PMG_TIMEOUT: return "timeout";
    case PMG_CUDA_ERR: return "CUDA error";
    case PMG_NOT_SPD: return "matrix not positive definite";
    default: return "unknown status";
  }
}

const char* pmg_last_error(void) { return pmg::last_error(); }

// Element stiffness K0 = sum_gp w B^T D B by 2x2(x2) Gauss quadrature at the points s * (h/2)/sqrt(3)
// (pymoto/modules/assembly.py:427-463, shape derivatives pymoto/common/domain.py:409-428,
// B pymoto/modules/assembly.py:318-370, D pymoto/modules/assembly.py:373-404).  Host-only.
int pmg_element_stiffness(int dim, double E, double nu, int plane_stress, double unitx, double unity, double unitz,
                          double* K0_host) {
  if ((dim != 2 && dim != 3) || !K0_host || !(unitx > 0) || !(unity > 0) || !(unitz > 0)) return PMG_BAD_ARG;
  const int nn = 1 << dim, nde = nn * dim, ns = dim == 3 ? 6 : 3;
  const double h[3] = {unitx, unity, unitz};
  // constitutive matrix
  double D[6][6] = {};
  const double mu = E / (2.0 * (1.0 + nu)), lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), c1 = 2.0 * mu + lam;
  if (dim == 3) {
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) D[a][b] = a == b ? c1 : lam;
    for (int a = 3; a < 6; ++a) D[a][a] = mu;
  } else if (plane_stress) {
    const double f = E / (1.0 - nu * nu);
    D[0][0] = f;
    D[0][1] = f * nu;
    D[1][0] = f * nu;
    D[1][1] = f;
    D[2][2] = f * (1.0 - nu) / 2.0;
  } else {
    D[0][0] = c1;
    D[0][1] = lam;
    D[1][0] = lam;
    D[1][1] = c1;
    D[2][2] = mu;
  }
  double vol = 1.0, w = 1.0;
  for (int a = 0; a < dim; ++a) {
    vol *= h[a];
    w *= h[a] / 2.0;
  }
  if (dim == 2) w *= h[2];
  for (int i = 0; i < nde * nde; ++i) K0_host[i] = 0.0;
  auto sgn = [](int node, int axis) { return ((node >> axis) & 1) ? 1.0 : -1.0; };
  for (int gp = 0; gp < nn; ++gp) {
    double pos[3];
    for (int a = 0; a < 3; ++a) pos[a] = (a < dim ? sgn(gp, a) : -1.0) * (h[a] / 2.0) / std::sqrt(3.0);
    double dN[3][8];
    for (int a = 0; a < dim; ++a)
      for (int n = 0; n < nn; ++n) {
        double v = 1.0 / vol;
        for (int b = 0; b < dim; ++b)
          if (b != a) v *= h[b] / 2.0 + sgn(n, b) * pos[b];
        dN[a][n] = v * sgn(n, a);
      }
    double B[6][24] = {};
    for (int n = 0; n < nn; ++n) {
      if (dim == 2) {
        B[0][2 * n] = dN[0][n];
        B[1][2 * n + 1] = dN[1][n];
        B[2][2 * n] = dN[1][n];
        B[2][2 * n + 1] = dN[0][n];
      } else {
        B[0][3 * n] = dN[0][n];
        B[1][3 * n + 1] = dN[1][n];
        B[2][3 * n + 2] = dN[2][n];
        B[3][3 * n + 1] = dN[2][n];
        B[3][3 * n + 2] = dN[1][n];
        B[4][3 * n] = dN[2][n];
        B[4][3 * n + 2] = dN[0][n];
        B[5][3 * n] = dN[1][n];
        B[5][3 * n + 1] = dN[0][n];
      }
    }
    double DB[6][24];
    for (int a = 0; a < ns; ++a)
      for (int q = 0; q < nde; ++q) {
        double v = 0.0;
        for (int b = 0; b < ns; ++b) v += D[a][b] * B[b][q];
        DB[a][q] = v;
      }
    for (int r = 0; r < nde; ++r)
      for (int c = 0; c < nde; ++c) {
        double v = 0.0;
        for (int a = 0; a < ns; ++a) v += B[a][r] * DB[a][c];
        K0_host[r * nde + c] += w * v;
      }
  }
  return PMG_OK;
}

}  // extern "C"
