/*
 * pymoto_gb300 -- C ABI of the GB300 (sm_103a) kernels for pyMOTO's structured-grid compliance path.
 *
 * Conventions
 *  - Grids are given by their element counts (nelx, nely, nelz); nelz == 0 selects the 2D (Q4, 2 dofs
 *    per node) path, nelz > 0 the 3D (hex8, 3 dofs per node) path.  Numbering is pyMOTO's:
 *    element (i,j,k) -> (k*nely + j)*nelx + i, node (i,j,k) -> (k*(nely+1) + j)*(nelx+1) + i,
 *    dof -> node*dim + d (pymoto/common/domain.py:200-251).
 *  - All array arguments are DEVICE pointers unless the name ends in _host.  `dtype` selects the
 *    storage type of the floating-point arrays: PMG_F64 or PMG_F32.  Reductions always accumulate in
 *    FP64 and write FP64 results.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are asynchronous and stream-
 *    ordered; none of them synchronises the device or allocates device memory.  Scratch buffers are
 *    passed in by the caller and their minimum sizes are given by the *_scratch_bytes queries.
 *  - Every call returns a pmg_status.  Invalid arguments are rejected before any launch.
 *  - `bcmask` is one byte per node; bit d set means dof (node, d) is a Dirichlet dof whose row and column
 *    are replaced by `bcdiag` on the diagonal (pymoto/modules/assembly.py:94-98, :210-230, :272).
 *  - Element matrices `K0_host` are row-major (2^dim*dim)^2 FP64 arrays in pyMOTO's local dof order.
 */
#ifndef PYMOTO_GB300_H
#define PYMOTO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PMG_OK = 0,
  PMG_BAD_ARG = 1,
  PMG_NOT_CONVERGED = 2,
  PMG_TIMEOUT = 3,
  PMG_CUDA_ERR = 4,
  PMG_NOT_SPD = 5
} pmg_status;

enum { PMG_F64 = 0, PMG_F32 = 1 };

/* Operator application modes for pmg_ebe_apply / pmg_stencil_apply. */
enum {
  PMG_APPLY_MATVEC = 0,   /* y = A u                                   */
  PMG_APPLY_RESIDUAL = 1, /* y = b - A u                               */
  PMG_APPLY_JACOBI = 2    /* y = u + omega * ((b - A u) / diag)        */
};

/* Library identification. */
int pmg_version(void);
const char* pmg_status_string(int status);
/* Last CUDA error string seen by the library in this thread (for PMG_CUDA_ERR). */
const char* pmg_last_error(void);

/* Element stiffness matrix (2^dim*dim)^2, row-major, of pyMOTO's AssembleStiffness (2x2(x2) Gauss
 * quadrature, replaces pymoto/modules/assembly.py:427-463).  dim 2 uses plane stress when
 * plane_stress != 0, else plane strain (pyMOTO's default); unitz is the 2D thickness.  Host-only. */
int pmg_element_stiffness(int dim, double E, double nu, int plane_stress, double unitx, double unity, double unitz,
                          double* K0_host);

/* ---- index maps ------------------------------------------------------------------------------
 * Dof connectivity (nel, 2^dim*dim) int64, bit-exact with VoxelDomain.get_dofconnectivity
 * (replaces pymoto/common/domain.py:338-362). */
int pmg_dof_connectivity(int nelx, int nely, int nelz, int64_t* dofconn, void* stream);

/* ---- matrix-free stiffness operator K(x) = sum_e x_e K0 (Dirichlet rows/cols -> bcdiag) --------
 * Replaces AssembleGeneral.__call__ (pymoto/modules/assembly.py:245-296) followed by the CSR products
 * of CG and GeometricMultigrid (pymoto/solvers/iterative.py:236-255, :375) and the damped-Jacobi
 * smoother (pymoto/solvers/iterative.py:41-47).  u, b, diag, y: ndof; xe: nel.  cdiag (ndof, or NULL): a
 * constant diagonal added to the operator after the Dirichlet rows are set, the diagonal add_constant of
 * AssembleGeneral (pymoto/modules/assembly.py:294-295): a Dirichlet row holds bcdiag + cdiag. */
int pmg_ebe_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                  const uint8_t* bcmask, double bcdiag, const void* u, const void* b, const void* diag,
                  double omega, void* y, const void* cdiag, void* stream);
/* diag(K(x)) (+ cdiag), replaces A.diagonal() of DampedJacobi.update (pymoto/solvers/iterative.py:38-39). */
int pmg_ebe_diagonal(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                     const uint8_t* bcmask, double bcdiag, void* diag, const void* cdiag, void* stream);

/* ---- assembled node-stencil operator of the coarse multigrid levels ---------------------------
 * The operators are symmetric, so S holds per node only the centre block and the blocks of the forward
 * offsets o > C, o = (dz+1)*9 + (dy+1)*3 + (dx+1) (3D, C = 13) or (dy+1)*3 + (dx+1) (2D, C = 4), in
 * structure-of-arrays order S[(h*dim + d)*dim + c][node] with h = o - C: 14 x 3 x 3 values per node in 3D,
 * 5 x 2 x 2 in 2D.  The block of a backward offset o < C at node n is the transpose of the block stored at
 * its neighbour n + off(o) for offset 2C - o.  Entries of offsets that leave the grid are zero.
 * Replaces the CSR products with the Galerkin operators R^T A R (pymoto/solvers/iterative.py:173,
 * :233-255). */
int pmg_stencil_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* S, const void* u,
                      const void* b, const void* diag, double omega, void* y, void* stream);
int pmg_stencil_diagonal(int dtype, int nelx, int nely, int nelz, const void* S, void* diag, void* stream);
/* Centre-block diagonal of S += c (ndof): a constant diagonal (add_constant, pymoto/modules/assembly.py:294-295)
 * on the level-0 stencils, and its restriction R^T c (a lumped Galerkin term) on the coarse levels. */
int pmg_stencil_add_diagonal(int dtype, int nelx, int nely, int nelz, void* S, const void* c, void* stream);

/* ---- grid transfers (trilinear / bilinear prolongation R of pymoto/solvers/iterative.py:178-220) --
 * Grid arguments are the FINE grid.  rc = R^T rf (iterative.py:244);  uf += R uc (iterative.py:250). */
int pmg_restrict(int dtype, int nelx, int nely, int nelz, const void* rf, void* rc, void* stream);
int pmg_prolong_add(int dtype, int nelx, int nely, int nelz, const void* uc, void* uf, void* stream);

/* ---- Galerkin coarse operators Ac = R^T A R (pymoto/solvers/iterative.py:173) -------------------
 * Computed per coarse element: E_C = sum_children M_c^T E_child M_c.  The coarse element matrices are
 * stored element-major, E[e][(2^dim*dim)^2].
 * pmg_galerkin_table fills the 2^dim host matrices M_c^T K0 M_c (the unconstrained children).
 * pmg_galerkin_from_ebe builds level-1 element matrices from the matrix-free fine operator; `table`
 * is the device copy of pmg_galerkin_table's output in the same dtype.
 * pmg_galerkin_from_elements builds the next level from element matrices (grid = the fine grid whose
 * elements Ef belongs to). */
int pmg_galerkin_table(int dim, const double* K0_host, double* table_host);
int pmg_galerkin_from_ebe(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                          const uint8_t* bcmask, double bcdiag, const void* table, const int32_t* bc_elems, int n_bc,
                          void* Ec, void* stream);
/* bc_elems (device, n_bc entries, or NULL): the coarse elements with a constrained fine node, which a second
 * launch handles one CTA each; with NULL they are found and handled inside the first launch. */
int pmg_galerkin_from_elements(int dtype, int nelx, int nely, int nelz, const void* Ef, void* Ec, void* stream);
/* Node stencils of a grid from its element matrices (assembly of sum_e P_e^T E_e P_e). */
int pmg_stencil_from_elements(int dtype, int nelx, int nely, int nelz, const void* E, void* S, void* stream);
/* Node stencils (same layout) of the level-0 operator K(x) with its Dirichlet rows/columns: K(x) assembled
 * once per design so that repeated products cost 3^dim*dim^2 FMA per node instead of the matrix-free
 * 2^dim*(2^dim*dim)*dim (the FP64 products of the solver; replaces the CSR data assembly of
 * pymoto/modules/assembly.py:245-296). */
int pmg_ebe_stencil(int dtype, int nelx, int nely, int nelz, const void* xe, const double* K0_host,
                    const uint8_t* bcmask, double bcdiag, void* S, void* stream);
/* Dense FP64 matrix (ndof x ndof, row-major) of a stencil operator: the coarsest-level system. */
int pmg_stencil_to_dense(int dtype, int nelx, int nely, int nelz, const void* S, double* A, void* stream);
/* The same in a permuted numbering: dof q goes to row/column pos[q] (pos == NULL: natural numbering). */
int pmg_stencil_to_dense_perm(int dtype, int nelx, int nely, int nelz, const void* S, const int32_t* pos, double* A,
                              void* stream);
/* Host-only: band-reducing numbering of the dofs of a grid (the axis with the fewest nodes fastest, the one with
 * the most slowest) into pos[ndof], and the half bandwidth *bw of a stencil matrix in that numbering.  On the
 * 9 x 5 x 5-node coarsest grid of a 128 x 64 x 64 hierarchy the band shrinks from 167 to 95, and the banded
 * Cholesky work (n bw^2 / 2) by 3x. */
int pmg_coarse_ordering(int nelx, int nely, int nelz, int32_t* pos, int* bw);
/* Half bandwidth of the dense coarsest matrix of a grid. */
int pmg_stencil_bandwidth(int nelx, int nely, int nelz);

/* ---- Chebyshev smoother (extends DampedJacobi, pymoto/solvers/iterative.py:21-47, with a polynomial
 * smoother on [lmax/ratio, lmax] of D^-1 A; Saad, Iterative Methods for Sparse Linear Systems, Alg. 12.1)
 * out (dof vector, operator dtype) = sum_j |A_ij| of a stencil operator: the l1-Jacobi diagonal, with
 * which lmax(D^-1 A) <= 1 by Gershgorin's theorem.  The matrix-free finest operator gets the same bound
 * from pmg_ebe_diagonal with K0 replaced by diag(sum_j |K0_aj|). */
int pmg_stencil_rowabs(int dtype, int nelx, int nely, int nelz, const void* S, void* out, void* stream);
/* coef[2j], coef[2j+1] (device, j < degree) = the step coefficients a_j, c_j for lmax = *lmax_dev (device
 * double) or lmax_host when lmax_dev is NULL. */
int pmg_cheb_coeffs(const double* lmax_dev, double lmax_host, double ratio, int degree, double* coef, void* stream);
/* Fused smoothing step on a stencil operator: r = b - A u computed in the product, d = a_j d + c_j r / dl1
 * (d not read at step 0), y = u + d (y != u). */
int pmg_stencil_cheb_step(int dtype, int nelx, int nely, int nelz, const void* S, const void* u, const void* b,
                          const void* dl1, void* d, const double* coef, int step, void* y, void* stream);
/* The same on the matrix-free FP32 3D level-0 operator (the kernel of pmg_ebe_apply). */
int pmg_ebe_cheb_step(int nelx, int nely, int nelz, const float* xe, const double* K0_host, const uint8_t* bcmask,
                      double bcdiag, const float* u, const float* b, const float* dl1, float* d, const double* coef,
                      int step, float* y, const float* cdiag, void* stream);
/* Status of the tensor-core operator kernels (pmg_ebe_apply / pmg_ebe_cheb_step on FP32 3D grids) since the
 * last reset (host-synchronous read): PMG_OK, or PMG_TIMEOUT if a bounded wait of a kernel gave up (its
 * output is then undefined).  reset != 0 clears the flag.  No counterpart in the reference: pyMOTO's
 * assembly has no device waits. */
int pmg_operator_status(int reset);
/* Implementation of the FP32 3D level-0 operator (pmg_ebe_apply, pmg_ebe_cheb_step): PMG_OPERATOR_FMA (default)
 * runs the element products as FP32 FMAs on the CUDA cores, one thread per node column; PMG_OPERATOR_TCGEN05 as
 * 3xTF32 products on the tensor cores (tcgen05.mma, accumulators in tensor memory).  Both give FP32-accurate
 * K(x) u.  Host only; returns the previous selection (kind = -1: the current one, unchanged), or -1 for an
 * unknown kind.  Process-wide: select before launching, not while another thread launches operator products. */
enum { PMG_OPERATOR_FMA = 0, PMG_OPERATOR_TCGEN05 = 1 };
int pmg_set_operator_kernel(int kind);
/* Host only: the launch plan of the CUDA-core FP32 3D operator for a grid and a number of resident CTA slots
 * (CTAs per SM x SMs): plan_host[0..4] = tile width OX and height OY in node columns, tiles in x and y, z chunks. */
int pmg_operator_plan(int nelx, int nely, int nelz, int slots, int* plan_host);
/* Step `step`: d = a d + c r / diag, x = x + d; init != 0 starts from x = 0 (d = x = c r / diag). */
int pmg_cheb_step(int dtype, int64_t n, const void* r, const void* diag, void* d, void* x, const double* coef, int step,
                  int init, void* stream);

/* ---- coarsest-level direct solve (replaces SolverSparseLU, pymoto/solvers/sparse.py:515-555, as
 * chosen by auto_determine_solver, pymoto/solvers/auto_determine.py:109-122) -----------------------
 * In-place FP64 Cholesky A = L L^T of a dense SPD matrix with half bandwidth `bw` (lower triangle
 * used).  `info` (device int) is set to 0, or to k+1 if the k-th pivot is not positive (that pivot is
 * replaced by 1 so the call always completes); the caller reads `info` once the stream has finished. */
int pmg_cholesky_factor(int n, double* A, int bw, int* info, void* stream);
/* x = (L L^T)^{-1} b.  L is FP64 or FP32 (dtype); b and x have the same dtype as L. */
int pmg_cholesky_solve(int dtype, int n, const void* L, int bw, const void* b, void* x, void* stream);
/* Ainv = (L L^T)^{-1} (dense, FP64, n x n): one CTA per row.  For the small coarsest level, whose solve is
 * then one dense matrix-vector product per V-cycle instead of two sequential substitutions. */
int pmg_cholesky_inverse(int n, const double* L, int bw, double* Ainv, void* stream);
/* Inverses of the TB x TB (TB = 32) diagonal tiles of the FP64 factor L, stored row-major one tile after
 * the other ((n+31)/32 tiles, zero-padded) in dtype FP64 or FP32: the operands of the blocked solve. */
int pmg_cholesky_block_inverses(int dtype, int n, const double* L, void* Dinv, void* stream);
/* x = (L L^T)^{-1} b by tiles: each tile of the forward and backward substitutions is one dense product
 * with its tile inverse, so the solve has no scalar recurrence (one CTA, x in shared memory).  L, Dinv, b
 * and x share the dtype; L is the banded factor (FP32 copy for FP32 right-hand sides). */
int pmg_cholesky_solve_blocked(int dtype, int n, const void* L, int bw, const void* Dinv, const void* b, void* x,
                               void* stream);
/* FP32 inverse Ainv = (L L^T)^{-1} (n x n, row-major) of the FP64 factor, for FP32 coarse solves by one
 * dense product: L^{-1} is formed in FP32 by tiles (tile inverses from the FP64 factor), then
 * Ainv = L^{-T} L^{-1}.  scratch >= pmg_cholesky_inverse_f32_scratch_bytes(n) bytes. */
size_t pmg_cholesky_inverse_f32_scratch_bytes(int n);
int pmg_cholesky_inverse_f32(int n, const double* L, int bw, void* scratch, float* Ainv, void* stream);
/* y = A x, dense row-major n x n, FP64 or FP32 storage with FP64 accumulation. */
int pmg_dense_gemv(int dtype, int n, const void* A, const void* x, void* y, void* stream);
/* out[i][j] = in[pos[i]][pos[j]] (n x n row-major, f64 or f32): returns a matrix computed in a permuted numbering
 * (pmg_stencil_to_dense_perm) to the natural one. */
int pmg_dense_permute(int dtype, int n, const int32_t* pos, const void* in, void* out, void* stream);

/* ---- reductions and vector updates of CG (pymoto/solvers/iterative.py:340-403) -----------------
 * Deterministic single-launch reductions with FP64 accumulation (CTA partials summed in CTA order by the
 * last CTA).  scratch >= pmg_reduce_scratch_bytes() bytes, zero-filled once before its first use; every
 * call leaves it ready for the next one.  Calls sharing one scratch buffer must be stream-ordered. */
size_t pmg_reduce_scratch_bytes(void);
/* out[0] = a.b */
int pmg_dot(int dtype, int64_t n, const void* a, const void* b, double* out, void* scratch, void* stream);
/* out[0] = a.b, out[1] = c.d in one pass */
int pmg_dot2(int dtype, int64_t n, const void* a, const void* b, const void* c, const void* d, double* out,
             void* scratch, void* stream);
/* out[0] = a.b without a scratch argument, for callers that cannot allocate device memory (for example
 * a plugin inside a host application that owns every device allocation).  This entry point has no
 * counterpart in the reference.  Its scratch is a static device array of about 32 KB held by every GPU that
 * loads the library; n is limited to 4,194,304 elements (larger n: PMG_BAD_ARG).  All calls on a device
 * share that array, so calls that overlap on the GPU race; calls ordered on one stream are safe.  The first
 * call in each CUDA context looks up the array's device address in that context; make it before any stream
 * capture.  Accumulation as pmg_dot (FP32 data: compensated FP32), over a different per-CTA split, so the
 * two agree to rounding, not bit for bit. */
int pmg_dot_noalloc(int dtype, int64_t n, const void* a, const void* b, double* out, void* stream);
/* In the *_ratio updates below a zero denominator gives a zero ratio (no update) instead of inf/nan. */
/* alpha = num[0]/den[0];  x += alpha p;  r -= alpha q;  rr_out[0] = r.r   (FP64 CG step). */
int pmg_cg_update(int dtype, int64_t n, void* x, void* r, const void* p, const void* q, const double* num,
                  const double* den, double* rr_out, void* scratch, void* stream);
/* x += scale * (num[0]/den[0]) p  (the explicit-residual iterations; scale -1 for projections). */
int pmg_axpy_ratio(int dtype, int64_t n, void* x, const void* p, const double* num, const double* den, double scale,
                   void* stream);
/* beta = -num[0]/den[0];  p = z + beta p. */
int pmg_xpby_ratio(int dtype, int64_t n, void* p, const void* z, const double* num, const double* den,
                   void* stream);
/* y = x * (1/sqrt(nrm2[0]))  (orth of a single vector, pymoto/solvers/iterative.py:259-292). */
int pmg_scale_rsqrt(int dtype, int64_t n, void* y, const void* x, const double* nrm2, void* stream);
/* y = a * x   (y, x of dtype), scalar a on the host. */
int pmg_scale(int dtype, int64_t n, void* y, const void* x, double a, void* stream);
/* y = x with the Dirichlet dofs zeroed (or only the Dirichlet dofs kept when keep_bc != 0).  dim: dofs per node
 * (1, 2 or 3; bit d of a node's mask byte marks its dof d), here and in pmg_split_bc. */
int pmg_mask_bc(int dtype, int dim, int64_t nnodes, const uint8_t* bcmask, int keep_bc, const void* x, void* y,
                void* stream);
/* One pass: direct = rhs / (bcdiag + cdiag) on the Dirichlet dofs (0 elsewhere; cdiag may be NULL), free_part =
 * rhs on the free dofs (0 on the Dirichlet dofs) -- the split of LDAWrapper.solve
 * (pymoto/solvers/solvers.py:174-176). */
int pmg_split_bc(int dtype, int dim, int64_t nnodes, const uint8_t* bcmask, double bcdiag, const void* rhs,
                 void* direct, void* free_part, const void* cdiag, void* stream);
/* Precision conversion y(dst_dtype) = a * x(src_dtype) (product formed in FP64); and x64 += a * d32. */
int pmg_convert(int src_dtype, int dst_dtype, int64_t n, const void* x, void* y, double a, void* stream);
int pmg_add_f32_to_f64(int64_t n, double* x, const float* d, double a, void* stream);
/* y = x * sqrt(s[0]) (inverse == 0) or x / sqrt(s[0]) (inverse != 0) with s a device scalar, e.g. the
 * squared residual norm: normalising a residual to the preconditioner's precision without a host read. */
int pmg_convert_dscale(int src_dtype, int dst_dtype, int64_t n, const void* x, void* y, const double* s, int inverse,
                       void* stream);
/* y = w * (b / diag): the first damped-Jacobi sweep from a zero guess (pymoto/solvers/iterative.py:233-234). */
int pmg_diag_scale(int dtype, int64_t n, const void* b, const void* diag, double w, void* y, void* stream);

/* ---- density filters (pymoto/modules/filter.py) --------------------------------------------------
 * DensityFilter (filter.py:223-378): y = H x / s, H_ij = max(0, r - |i-j|) over the window int(r).
 * `transpose` != 0 computes H (x / s).  s (nel) is written by pmg_density_filter_rowsum. */
int pmg_density_filter_rowsum(int nelx, int nely, int nelz, double radius, double* s, void* stream);
int pmg_density_filter(int transpose, int nelx, int nely, int nelz, double radius, const double* s,
                       const double* x, double* y, void* stream);
/* FilterConv (filter.py:8-220) with per-axis padded index maps pad{x,y,z} (int32, length n+2p, device)
 * and kernel weights w (kx*ky*kz, C order, device).  Forward: y = W * x_pad ('valid', filter.py:207-212).
 * A map entry -1 marks a padded position of a constant-value side: it contributes nothing, and the caller
 * adds the constant values' field (linear in the constants, fixed per filter). */
int pmg_conv_filter(int nelx, int nely, int nelz, const double* w, int kx, int ky, int kz, const int32_t* padx,
                    const int32_t* pady, const int32_t* padz, const double* x, double* y, void* stream);
/* Its adjoint (filter.py:214-220: full correlation accumulated through the pad maps), with the inverse pad
 * maps: the padded positions of index j along an axis are inv_pos[inv_ptr[j] .. inv_ptr[j+1]). */
int pmg_conv_filter_adjoint(int nelx, int nely, int nelz, const double* w, int kx, int ky, int kz,
                            const int32_t* invx_ptr, const int32_t* invx_pos, const int32_t* invy_ptr,
                            const int32_t* invy_pos, const int32_t* invz_ptr, const int32_t* invz_pos,
                            const double* d, double* y, void* stream);

/* ---- SIMP interpolation (MathExpression "xmin + (1-xmin) x^p", pymoto/modules/generic.py:94-140) -- */
int pmg_simp(int64_t n, double xmin, double penal, const double* x, double* y, void* y32, void* stream);
/* dx = dy * p (1-xmin) x^(p-1) */
int pmg_simp_backward(int64_t n, double xmin, double penal, const double* x, const double* dy, double* dx,
                      void* stream);

/* ---- adjoint sensitivity contraction (pymoto/modules/assembly.py:298-315 with
 * DyadicMatrix.contract, pymoto/common/dyadcarrier.py:366-414) ------------------------------------
 * dx_e (+)= alpha * u_e^T K0 v_e with Dirichlet entries of u and v zeroed (dyadcarrier.py:179-189). */
int pmg_sens_contract(int nelx, int nely, int nelz, const double* K0_host, const uint8_t* bcmask,
                      const double* u, const double* v, double alpha, int accumulate, double* dx, void* stream);
/* The same contraction for the mixed-precision path: element vectors shifted in FP64 by their first-node
 * value (exact: K0 annihilates translations), the quadratic form in FP32, the result in FP64. */
int pmg_sens_contract_mixed(int nelx, int nely, int nelz, const double* K0_host, const uint8_t* bcmask,
                            const double* u, const double* v, double alpha, int accumulate, double* dx,
                            void* stream);

/* ---- optimality-criteria update (OC.step, pymoto/common/optimizers.py:402-437) -----------------
 * Bisection on the Lagrange multiplier fully on the device; xnew is the design of the last bisection
 * step.  scratch >= pmg_oc_scratch_bytes(). */
size_t pmg_oc_scratch_bytes(void);
int pmg_oc_update(int64_t n, const double* x, const double* dg, double* xnew, double volfrac, double move,
                  double xmin, double xmax, double l1, double l2, double l1l2tol, void* scratch, void* stream);
/* Status of the last pmg_oc_update on `scratch` (host-synchronous read): PMG_OK, or PMG_TIMEOUT if a
 * bounded wait of the single-launch bisection expired (its CTAs were not all resident). */
int pmg_oc_status(const void* scratch);
/* Test control of the bounded device waits of the OC update (host-synchronous): every wait gives up after
 * `polls` polls (0: the built-in limit of a few seconds), and with withhold_arrival != 0 the last CTA of the
 * grid-wide barrier withholds its arrival, so that the waits run out; the update then ends with PMG_TIMEOUT in
 * pmg_oc_status.  For tests of the failure path; no counterpart in the reference (pyMOTO's OC has no device
 * waits). */
int pmg_set_wait_test(unsigned polls, int withhold_arrival);
/* The same status word copied into host memory (`status`, pinned for an asynchronous copy) in stream order:
 * nonzero once the copy has completed means the bisection's bounded wait expired.  Lets a host loop read
 * the status at its next synchronisation instead of adding one. */
int pmg_oc_status_async(const void* scratch, unsigned* status, void* stream);

/* ---- additive-manufacturing overhang filter (OverhangFilter, pymoto/modules/filter.py:381-713) ---------------
 * One launch per layer `layer` along the print axis `lay` (0 x, 1 y, 2 z), print direction `step` (+1 / -1);
 * nz >= 1 (a 2D grid passes nz = 1).  The K support kernels kern[K][w0][w1][w2] (C order) span one layer (w_lay
 * = 1) and an odd window in the other axes, centred: c_lay = step, c_other = (w - 1) / 2.  Forward (layers in
 * print order): s = (sum_k (v_k + shift)^p)^(1/q) - backshift over the previous printed layer (a baseplate of 1
 * below the first), y = smooth min of x and s.  Adjoint (layers in reverse print order, `first` for the first
 * call): dx from dy; the derivatives of this layer's supports go to dsupp_cur[K][plane], those of the layer
 * processed before are read from dsupp_later (two distinct buffers, swapped between calls). */
int pmg_overhang_forward(int nx, int ny, int nz, int lay, int step, int layer, int w0, int w1, int w2, int c0, int c1,
                         int c2, int K, const double* kern, double p, double q, double shift, double backshift,
                         double eps, const double* x, double* y, double* s, void* stream);
int pmg_overhang_adjoint(int nx, int ny, int nz, int lay, int step, int layer, int first, int w0, int w1, int w2,
                         int c0, int c1, int c2, int K, const double* kern, double p, double q, double shift,
                         double backshift, double eps, const double* x, const double* y, const double* s,
                         const double* dy, double* dsupp_cur, const double* dsupp_later, double* dx, void* stream);

/* ---- Method of Moving Asymptotes (MMA.step / mmasub / subsolv, pymoto/common/mma.py:96-474) ----------
 * One design update: the asymptote offsets adapt from xold1/xold2 (when params.adapt), the convex separable
 * approximation is built from the responses g[m+1] and their sensitivities dg[(m+1) x n] (row-major; row 0 the
 * objective), and its subproblem is solved by the primal-dual Newton method down to params.epsimin (already
 * scaled by sqrt(m + n)), all in one cooperative launch (plus a reset and a status kernel).  The unconstrained
 * problem is passed with pyMOTO's dummy constraint (g = -1, zero sensitivities).  xmin, xmax, move are
 * per-variable arrays; offset is updated in place; low/upp receive the asymptotes, xnew the new design and
 * info (device, m + 6 doubles): gest[0..m], dk, status (0 ok, 1 a bounded wait expired, 2 singular Newton
 * system), epsilon levels, Newton iterations, line-search trials.  scratch >= pmg_mma_scratch_bytes(n, m). */
#define PMG_MMA_MAX_M 4
enum { PMG_MMA_1987 = 0, PMG_MMA_2007 = 1, PMG_MMA_GCMMA = 2 };
typedef struct {
  int version;   /* PMG_MMA_1987, PMG_MMA_2007 or PMG_MMA_GCMMA */
  int m;         /* general constraints, 1..PMG_MMA_MAX_M */
  int adapt;     /* adapt the asymptote offsets from xold1, xold2 */
  int maxit;     /* Newton and line-search iteration limit (pyMOTO: 400) */
  int exact;     /* 1: divide wherever pyMOTO divides (numpy's rounding); 0: one reciprocal per denominator */
  int reserved;  /* 0 */
  double a0, albefa, asyincr, asydecr;
  double offmin, offmax;          /* offset clip: 1/asybound^2, asybound */
  double epsimin;                 /* epsimin * sqrt(m + n) */
  double rho[PMG_MMA_MAX_M + 1];  /* MMA2007: rho[0]; GCMMA: one per response */
  double a[PMG_MMA_MAX_M], c[PMG_MMA_MAX_M], d[PMG_MMA_MAX_M];
} pmg_mma_params;
size_t pmg_mma_scratch_bytes(int64_t n, int m);
int pmg_mma_update(int64_t n, const pmg_mma_params* params_host, const double* xval, const double* xold1,
                   const double* xold2, const double* xmin, const double* xmax, const double* move, const double* g,
                   const double* dg, double* offset, double* low, double* upp, double* xnew, double* info,
                   void* scratch, void* stream);

/* ---- learned warm start (no counterpart in the reference: the reference solves every design from the
 * previous solution only).  A 3-level convolutional encoder-decoder on the voxel grid of a coarse
 * multigrid level, trained on the device on (density, displacement) pairs of the solver.  Layout
 * channels-last act[v][c], v = (k*ny + j)*nx + i; activations and weights BF16, accumulation and gradients
 * FP32, weights w[tap][cin][cout] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1), zero padding. -------------- */
/* out[v][co] = bias[co] + sum w in (+ ReLU); `in` BF16 (or FP32 if in_is_f32); out_bf16 and/or out_f32. */
int pmg_nn_conv3d_forward(int nx, int ny, int nz, int cin, int cout, int in_is_f32, const void* in, const void* w,
                          const float* bias, int relu, void* out_bf16, float* out_f32, void* stream);
/* din = conv^T(dout) (FP32). */
int pmg_nn_conv3d_backward_data(int nx, int ny, int nz, int cin, int cout, const float* dout, const void* w, float* din,
                                void* stream);
/* dw_db[27*cin*cout + cout] (+)= weight and bias gradients; scratch >= pmg_nn_wgrad_scratch_bytes(). */
size_t pmg_nn_wgrad_scratch_bytes(int nx, int ny, int nz, int cin, int cout);
int pmg_nn_conv3d_backward_weights(int nx, int ny, int nz, int cin, int cout, int in_is_f32, const void* in,
                                   const float* dout, float* dw_db, int accumulate, void* scratch, void* stream);
/* d *= (act > 0) for the stored BF16 ReLU output act. */
int pmg_nn_relu_backward(int64_t n, const void* act_bf16, float* d, void* stream);
/* 2x average pooling onto the coarse grid cnx x cny x cnz (direction 0, BF16), or its adjoint (direction 1,
 * FP32, adding into the fine gradient). */
int pmg_nn_pool2(int direction, int cnx, int cny, int cnz, int c, const void* in, void* out, void* stream);
/* 2x nearest upsampling of c channels into channels [coff, coff+c) of a ctot-channel fine tensor
 * (direction 0, BF16), or its adjoint (direction 1, FP32). */
int pmg_nn_up2(int direction, int cnx, int cny, int cnz, int c, int ctot, int coff, const void* in, void* out,
               void* stream);
/* out[v][coff + ch] = in[v][ch] (BF16) and the adjoint dskip[v][ch] += dcat[v][coff + ch] (FP32). */
int pmg_nn_copy_channels(int64_t nvox, int c, int ctot, int coff, const void* in, void* out, void* stream);
int pmg_nn_split_channels(int64_t nvox, int c, int ctot, int coff, const float* dcat, float* dskip, void* stream);
/* Input features on the voxel grid of stride `stride`: mean cube root of the element stiffness scaling xe
 * (mapped to [-1,1]) and voxel coordinates. */
int pmg_nn_input_features(int nelx, int nely, int nelz, int stride, int vnx, int vny, int vnz, const double* xe,
                          void* feat, void* stream);
/* Nodal field (FP64, 3 components) averaged from voxel values (direction 0), or the adjoint from FP32 nodal
 * gradients to FP32 voxel gradients (direction 1). */
int pmg_nn_vox_to_node(int direction, int vnx, int vny, int vnz, const void* in, void* out, void* stream);
/* Adam step (step >= 1) on FP32 master weights, refreshing their BF16 copy (if not NULL). */
int pmg_nn_adam(int n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr, float beta1, float beta2,
                float eps, int step, float weight_decay, void* stream);
/* loss_partial[block] = weight * sum (pred - target)^2 over the block; grad = 2 weight (pred - target). */
int pmg_nn_mse(int64_t n, const double* pred, const double* target, double weight, float* grad, double* loss_partial,
               void* stream);
/* uc = scale * u_f at every stride-th node of the fine grid (3 components). */
int pmg_nn_inject(int nelx, int nely, int nelz, int stride, const double* uf, double scale, double* uc,
                  void* stream);

/* ---- One-component operators (one dof per node): AssemblePoisson and AssembleMass with ndof = 1
 * (pymoto/modules/assembly.py:466-560; the CSR matrix of AssembleGeneral, assembly.py:245-296, and the
 * multigrid of pymoto/solvers/iterative.py:124-256 for it).  Node stencils are stored in full: S[o * nnodes + n]
 * (dtype) is the coefficient of node n towards its neighbour at offset o = (dz+1)*9 + (dy+1)*3 + (dx+1)
 * (27 offsets in 3D, 9 in 2D), zero for neighbours outside the grid.
 * Level 0: S = sum_e xe_e P0 (xe FP64 per element, P0 the host FP64 element matrix of 2^dim nodes in the local
 * order of pymoto/common/domain.py:132-142), accumulated in FP64; a node with bit 0 of bcmask set has bcdiag on
 * its diagonal and nothing else in its row and column; cdiag (FP64 per node, or NULL) is added to the diagonal. */
int pmg_scalar_stencil(int dtype, int nelx, int nely, int nelz, const double* xe, const double* P0_host,
                       const uint8_t* bcmask, double bcdiag, const double* cdiag, void* S, void* stream);
/* y = S u (mode PMG_APPLY_MATVEC), b - S u (PMG_APPLY_RESIDUAL) or u + omega (b - S u) / diag
 * (PMG_APPLY_JACOBI); y != u. */
int pmg_scalar_apply(int mode, int dtype, int nelx, int nely, int nelz, const void* S, const void* u, const void* b,
                     const void* diag, double omega, void* y, void* stream);
/* rc = R^T rf and uf += R uc with the (bi/tri)linear prolongation R of the grid of nelx x nely x nelz elements
 * (even counts) onto its coarse grid: weights 1, 1/2, 1/4, 1/8 (pymoto/solvers/iterative.py:182-189). */
int pmg_scalar_restrict(int dtype, int nelx, int nely, int nelz, const void* rf, void* rc, void* stream);
int pmg_scalar_prolong_add(int dtype, int nelx, int nely, int nelz, const void* uc, void* uf, void* stream);
/* Galerkin coarse operator Sc = R^T Sf R (pymoto/solvers/iterative.py:173), stencil to stencil, FP64
 * accumulation for FP64 operators, FP32 for FP32 ones; the grid is the fine one. */
int pmg_scalar_galerkin(int dtype, int nelx, int nely, int nelz, const void* Sf, void* Sc, void* stream);
/* Dense FP64 matrix (nnodes x nnodes, row-major, nnodes <= 65536) of a one-component operator. */
int pmg_scalar_to_dense(int dtype, int nelx, int nely, int nelz, const void* S, double* A, void* stream);
/* d = sum_o |S(n, o)|: the l1-Jacobi diagonal of the Chebyshev smoother. */
int pmg_scalar_rowabs(int dtype, int nelx, int nely, int nelz, const void* S, void* d, void* stream);
/* dx_e (+= when accumulate) alpha u_e^T P0 v_e (FP64) with the Dirichlet nodes of u and v taken as zero: the
 * design sensitivity of the assembled matrix contracted with the dyad (u, v) (assembly.py:298-315). */
int pmg_scalar_sens(int nelx, int nely, int nelz, const double* P0_host, const uint8_t* bcmask, const double* u,
                    const double* v, double alpha, int accumulate, double* dx, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PYMOTO_GB300_H */
