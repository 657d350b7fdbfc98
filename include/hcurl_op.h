/*
 * hcurl_op.h -- C ABI of the GB300 H(curl) curl-curl + mass operator and solver.
 *
 * One handle owns one discretised problem on the device: the Nedelec space on
 * a structured hex grid (sum-factorised partial assembly) or on a tet mesh
 * (closed-form FP64 element matrices, orders 1-2), the per-element
 * coefficient factors, the essential
 * (tangential Dirichlet) dof set and all Krylov work space.  The operator is
 * the reference's A/E-formulation bilinear form
 *
 *     a1(u, u') = (sigma u, u') + (dt nu curl u, curl u')
 *
 * (src/formulations/HCurl/hcurl_formulation.cpp:1-38), i.e. the sum of the
 * contributions that CurlCurlKernel (src/kernels/curl_curl_kernel.cpp:21-24,
 * coefficient dt*alpha registered at hcurl_formulation.cpp:117-128) and
 * VectorFEMassKernel (src/kernels/vector_fe_mass_kernel.cpp:21-24) add to the
 * ParBilinearForm.  "Mult" entry points apply the operator after essential-dof
 * elimination, exactly what EquationSystem::Mult / GetGradient expose
 * (src/equation_systems/equation_system.cpp:133-210):
 *
 *     J x = P K P x + (I - P) x,     P = projector onto non-essential dofs.
 *
 * Conventions
 *  - No call aborts or throws.  Every call returns hc_status; on failure
 *    hc_last_error() gives a one-line reason (thread-local for hc_create).
 *  - Host-pointer calls (hc_mult, hc_solve, ...) copy in, run on the
 *    handle's stream and synchronise; they are what an mfem::Operator /
 *    mfem::Solver shim calls with Vector::HostRead()/HostWrite() data.
 *  - *_device calls take device pointers, enqueue on the handle's stream and
 *    return without synchronising.
 *  - A handle is not re-entrant; different handles may be used from
 *    different host threads on different streams.
 *  - Dof numbering of the structured hex space (see hc_hex_dof_index) is
 *    tensor-product: component c's dofs are open (Gauss-Legendre nodal) in
 *    direction c and closed (Gauss-Lobatto nodal) in the other two, x
 *    fastest, components concatenated.
 */
#ifndef HCURL_OP_H
#define HCURL_OP_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hcop hcop_t;

typedef enum {
  HC_OK = 0,
  HC_EINVAL = 1,         /* bad argument (null pointer, size, NaN, ...)   */
  HC_ENOMEM = 2,         /* device allocation failed / over HBM budget    */
  HC_ECUDA = 3,          /* CUDA runtime error                            */
  HC_NOT_CONVERGED = 4,  /* maxit reached                                 */
  HC_BREAKDOWN = 5,      /* p^T K p <= 0, NaN or Inf in the iteration     */
  HC_TIMEOUT = 6,        /* a bounded device wait expired                 */
  HC_ENOTSUP = 7         /* valid request this build does not support     */
} hc_status;

enum { HC_HEX = 0, HC_TET = 1 };

/* Precision of a solve or of a device apply. */
enum {
  HC_FP64 = 0,   /* plain FP64 operator and PCG (the drop-in path)        */
  HC_FP32 = 1,   /* FP32 operator and vectors, FP64 dots and alpha/beta   */
  HC_MIXED = 2,  /* FP32 inner PCG inside FP64 iterative refinement       */
  HC_BF16 = 3,   /* tet multi-RHS apply: BF16 element matrices, FP32
                    vectors and accumulation                               */
  HC_MIXED_RR = 4 /* one FP32 PCG (COCG for complex solves) whose recursive
                    residual is replaced by the FP64 residual b - J x (and
                    its correction added to the FP64 x) each time it fell
                    by inner_rtol (per column in block solves); real,
                    block and complex solves (complex ones run the
                    graph-driven solve)                                    */
};

/* HC_PRECOND_AUX: Jacobi plus the auxiliary-space gradient correction
 * G V G^T (V one multigrid V-cycle for G^T M_sigma G on the H1 nodes), the
 * gradient part of the AMS preconditioner the reference uses
 * (hcurl_formulation.cpp:69-79).  Structured hex grids with sigma.
 * HC_PRECOND_AUX_MULT (hex handles, real solves): the same correction in a
 * symmetric multiplicative cycle, z = S r; z += c G V G^T (r - J z);
 * z += S (r - J z), S the Chebyshev-Jacobi polynomial of degree cheb_degree
 * (<= 0 -> 2) on [lmax/cheb_ratio, lmax], c = 1/2: 2 cheb_degree operator
 * applications per iteration, several times fewer iterations.  With
 * HC_MIXED_RR it suits tolerances down to about 1e-10; tighter ones reach
 * the FP32 floor of high-contrast fields and fall back to FP64 polishing. */
enum { HC_PRECOND_NONE = 0, HC_PRECOND_JACOBI = 1, HC_PRECOND_CHEBYSHEV = 2, HC_PRECOND_AUX = 3,
       HC_PRECOND_AUX_MULT = 4 };

typedef struct {
  int32_t elem_type;        /* HC_HEX (structured grid) or HC_TET                 */
  int32_t order;            /* Nedelec order: hex 1..3, tet 1..2                  */
  /* HC_HEX */
  int32_t nx, ny, nz;       /* elements per direction                             */
  /* HC_TET */
  int64_t n_vert;           /* vertex count                                       */
  int64_t n_elem;           /* tet count                                          */
  const int64_t* elem_verts;/* n_elem * 4 vertex ids                              */
  /* both */
  const double* vertices;   /* HC_HEX: (nx+1)(ny+1)(nz+1)*3, x fastest, NULL =
                               unit cube; every hex must be a parallelepiped.
                               HC_TET: n_vert*3                                    */
  const double* nu;         /* per-element curl-curl coefficient (required, >= 0)  */
  const double* sigma;      /* per-element mass coefficient (>= 0), NULL = none    */
  double dt;                /* curl-curl scale: K = dt*C_nu + M_sigma (> 0)        */
  /* essential (tangential Dirichlet) dofs: explicit mask wins over attributes */
  const uint8_t* ess_mask;  /* n_dof flags or NULL                                 */
  int32_t ess_attr_bits;    /* bit a-1 marks boundary attribute a.  HC_HEX faces:
                               1..6 = x-, x+, y-, y+, z-, z+.                      */
  int64_t n_bdr;            /* HC_TET boundary triangles                           */
  const int64_t* bdr_tris;  /* n_bdr * 3 vertex ids                                */
  const int32_t* bdr_attr;  /* n_bdr attributes                                    */
} hc_problem_desc;

typedef struct {
  int32_t precision;        /* HC_FP64 | HC_FP32 | HC_MIXED                        */
  int32_t precond;          /* HC_PRECOND_*                                        */
  int32_t cheb_degree;      /* polynomial degree (>= 1) for HC_PRECOND_CHEBYSHEV,
                               smoother degree of HC_PRECOND_AUX_MULT (<= 0 -> 2) */
  double cheb_ratio;        /* interval [lmax/ratio, lmax]; <= 0 -> 30              */
  double cheb_lmax;         /* upper eigenvalue bound of D^-1 J; <= 0 -> estimate  */
  double rtol, atol;        /* stop when ||b - J x|| <= max(rtol ||b||, atol)      */
  int32_t maxit;            /* max PCG iterations (inner iterations in total)      */
  double inner_rtol;        /* HC_MIXED: inner FP32 solve tolerance (<= 0 -> 1e-4);
                               HC_MIXED_RR: residual reduction between
                               replacements (<= 0 -> 0.1, capped at 0.5)      */
  int32_t max_outer;        /* HC_MIXED: max refinement steps (<= 0 -> 50)          */
} hc_solve_params;

typedef struct {
  int32_t status;           /* hc_status of the solve                              */
  int32_t iterations;       /* total PCG iterations                                */
  int32_t outer_iterations; /* refinement steps (HC_MIXED), residual replacements
                               (HC_MIXED_RR), else 1                           */
  int32_t applies;          /* operator applications                               */
  double rel_residual;      /* ||b - J x||_2 / ||b||_2 in FP64 at exit             */
  double lmax;              /* Chebyshev upper bound used                          */
} hc_solve_info;

/* ---- lifecycle ---------------------------------------------------------- */
/* Replaces the construction of CurlCurlEquationSystem's bilinear form +
 * FormLinearSystem (equation_system.cpp:133-198, 325-347): all inputs are
 * copied to the device, coefficient factors are computed in FP64.           */
hc_status hc_create(const hc_problem_desc* desc, hcop_t** out);
void hc_destroy(hcop_t* h);
/* Stream for all later work of this handle (cudaStream_t; NULL = default). */
hc_status hc_set_stream(hcop_t* h, void* stream);
/* Last error of this handle, or of the calling thread's last hc_create when
 * h is NULL.                                                               */
hc_status hc_last_error(const hcop_t* h, char* buf, size_t n);

/* ---- sizes / layout ----------------------------------------------------- */
int64_t hc_num_dofs(const hcop_t* h);
int64_t hc_num_elems(const hcop_t* h);
/* Structured hex: global index of dof (component c, i, j, k).             */
int64_t hc_hex_dof_index(const hcop_t* h, int c, int64_t i, int64_t j, int64_t k);
/* Essential-dof mask as the library resolved it (n_dof bytes, host).      */
hc_status hc_get_ess_mask(const hcop_t* h, uint8_t* mask);

/* ---- operator actions ---------------------------------------------------- */
/* y = J x (eliminated operator), host FP64 vectors.
 * Replaces EquationSystem::Mult (equation_system.cpp:201-204).              */
hc_status hc_mult(hcop_t* h, const double* x, double* y);
/* y = K x (full form, no elimination), host FP64.                          */
hc_status hc_apply_form(hcop_t* h, const double* x, double* y);
/* y += scale * C_nu x (curl-curl with nu alone, no dt, no elimination):
 * WeakCurlCurlKernel::Apply's _curl_curl->AddMultTranspose(u, lf, -1)
 * (src/kernels/weak_curl_curl_kernel.cpp:27-31) with scale = -1.            */
hc_status hc_add_weak_curlcurl(hcop_t* h, const double* x, double* y, double scale);
hc_status hc_add_weak_curlcurl_device(hcop_t* h, const double* x, double* y, double scale);
/* Diagonal of J (HypreDiagScale's diagonal, hephaestus_solvers.hpp:34-57).  */
hc_status hc_diag(hcop_t* h, double* d);

/* Launch configuration of the tiled hex kernels (orders 1-2): brick shape
 * 0 = 16x4x2 elements per CTA, 1 = 8x8x2; per_sm = CTAs per SM of the
 * persistent grid (0 = the launcher's choice, larger values are capped by
 * the occupancy).  Results do not depend on it beyond rounding order.     */
hc_status hc_set_launch(hcop_t* h, int32_t shape, int32_t per_sm);
hc_status hc_get_launch(const hcop_t* h, int32_t* shape, int32_t* per_sm);
/* Autotuner: times the FP32 apply (kind 0: the masked real apply of the
 * inner PCG iterations; 1: the fused complex apply of COCG) for each brick
 * shape and per_sm in 0..4 with CUDA events on the handle's stream (two
 * warm-up and five timed launches each) and keeps the fastest for this
 * handle.  The choice is also kept in a process-wide table keyed by (order,
 * grid, axis-aligned or not) and, when the environment variable
 * HC_TUNE_FILE names a file, appended to it; hc_create applies a stored
 * entry for its key.  Outputs (may be NULL): the chosen shape and per_sm,
 * the mean launch time of the choice and of the default (0, 0) in us.
 * HC_ENOTSUP for tet handles and hex order 3 (no tiled kernel).           */
hc_status hc_autotune(hcop_t* h, int32_t kind, int32_t* shape, int32_t* per_sm, double* us_best,
                      double* us_default);

/* Device-pointer forms, enqueued on the handle's stream.                   */
hc_status hc_mult_device(hcop_t* h, const double* x, double* y);
hc_status hc_mult_device_f32(hcop_t* h, const float* x, float* y);
hc_status hc_apply_form_device(hcop_t* h, const double* x, double* y);
/* y += P K P x (no initialisation of y; MFEM Operator::AddMult of the
 * eliminated form without its identity block).  One kernel launch.        */
hc_status hc_add_mult_device(hcop_t* h, const double* x, double* y);
hc_status hc_add_mult_device_f32(hcop_t* h, const float* x, float* y);

/* ---- around the solve ---------------------------------------------------- */
/* B = curl A into the Raviart-Thomas space of the grid (CurlAuxSolver with
 * MFEM's CurlInterpolator, src/auxsolvers/curl_aux.cpp:13-30).  Component c
 * is closed (Gauss-Lobatto nodal) in direction c and open (Gauss-Legendre
 * nodal) in the other two; layout as hc_hex_rt_dof_index.  B is the
 * reference-element flux: B_phys = J B_ref / det J at a point.             */
int64_t hc_num_rt_dofs(const hcop_t* h);
int64_t hc_hex_rt_dof_index(const hcop_t* h, int c, int64_t i, int64_t j, int64_t k);
hc_status hc_curl(hcop_t* h, const double* A, double* B);
hc_status hc_curl_device(hcop_t* h, const double* A, double* B);
/* hc_curl without any device allocation in the call: B is staged in a static
 * device area of HC_CURL_STATIC_MAX_RT_DOFS doubles (8 MiB) instead of a
 * buffer allocated per call.  Grids with more Raviart-Thomas dofs return
 * HC_EINVAL.  The first call on each device looks the area up with
 * cudaGetSymbolAddress (make it before any stream capture).  The area is
 * shared by every caller on a device: calls that overlap in time there race
 * and must be serialised.  No counterpart in the reference.               */
#define HC_CURL_STATIC_MAX_RT_DOFS (1 << 20)
hc_status hc_curl_static(hcop_t* h, const double* A, double* B);

/* Loop coil J = I0 (-(y-yc), x-xc, 0) for r0 <= r <= r1, z0 <= z <= z1 (r about
 * (xc, yc)), else 0.  b_i = (J, w_i) with a q^3 Gauss-Legendre rule per hex,
 * or the q^3 collapsed (Duffy) Gauss-Legendre rule per tet (1 <= q <= 8):
 * the right-hand side DivFreeSource adds
 * (src/sources/div_free_source.cpp:72-114).                                  */
typedef struct {
  double I0, xc, yc, r0, r1, z0, z1;
} hc_coil;
hc_status hc_load_coil(hcop_t* h, const hc_coil* coil, int q, double* b);
hc_status hc_load_coil_device(hcop_t* h, const hc_coil* coil, int q, double* b);

/* Y = J X for nrhs right-hand sides stored row-major ([dof][rhs]), device
 * pointers of the given precision (HC_FP64: double, HC_FP32 and HC_BF16:
 * float; HC_BF16 reads element matrices rounded to BF16, tets only);
 * nrhs in {1, 2, 4, 8, 16, 32}.  Tet meshes apply each element matrix to all
 * right-hand sides at once (one element-matrix read serves every column). */
hc_status hc_mult_multi_device(hcop_t* h, int precision, int nrhs, const void* X, void* Y);
/* HC_HEX or HC_TET */
int32_t hc_elem_type(const hcop_t* h);
/* Tet meshes: the FP64 element matrix (L x L, L = 6 or 20) of element e,
 * rows/columns in the local dof order of the basis.                        */
hc_status hc_tet_element_matrix(hcop_t* h, int64_t e, double* out);
/* y = G u: the discrete gradient from P1 vertex values u (n_vert device
 * doubles) into this Nedelec space (ndof device doubles), the G that HypreAMS
 * takes (MFEM's DiscreteLinearOperator with a GradientInterpolator); exact:
 * curl(G u) = 0.  Tet meshes.                                              */
hc_status hc_tet_gradient_device(hcop_t* h, const double* u, double* y);
/* Solve J X = B for nrhs right-hand sides together (block PCG with Jacobi,
 * one batched element-matrix apply per iteration for all columns), device
 * pointers in the [dof][rhs] layout of hc_mult_multi_device; X holds the
 * initial guesses.  Each column keeps its own alpha, beta and stopping test
 * (max(rtol ||b_k||, atol)); a converged column is frozen while the others
 * continue.  HC_FP64, or HC_MIXED: FP32 inner block PCG on column-normalised
 * residuals inside FP64 iterative refinement, with an FP64 block PCG from
 * the refined X when a refinement step stops cutting the residuals.  info
 * holds nrhs reports; returns the first non-OK column status.  Tet meshes;
 * nrhs in {1, 2, 4, 8, 16, 32}; precond HC_PRECOND_JACOBI, or
 * HC_PRECOND_AUX: Jacobi plus the gradient-space correction (PG) V (PG)^T
 * with V one V-cycle of a smoothed-aggregation AMG on the P1 nodal operator
 * (PG)^T J (PG), applied to all columns at once (hc_solve / hc_solve_device
 * with HC_PRECOND_AUX on a tet mesh run this with nrhs = 1).  B and X must
 * be 16-byte aligned (cudaMalloc and PyTorch allocations are).  Replaces R
 * separate HyprePCG solves of the same operator
 * (hcurl_formulation.cpp:81-85, problem_builder_base.cpp:221-253).        */
hc_status hc_solve_multi_device(hcop_t* h, const hc_solve_params* prm, int32_t nrhs, const double* B, double* X,
                                hc_solve_info* info);
/* hc_solve_multi_device with host arrays (same [dof][rhs] layout; X holds
 * the initial guesses and receives the solutions).                         */
hc_status hc_solve_multi(hcop_t* h, const hc_solve_params* prm, int32_t nrhs, const double* B, double* X,
                         hc_solve_info* info);
/* Tet auxiliary-space preconditioner, once set up by an HC_PRECOND_AUX solve:
 * returns the number of AMG levels and writes their sizes (free vertices on
 * level 0) to sizes[0..], followed by the number of free edge bubbles when
 * max_levels allows; 0 before set-up.                                       */
int32_t hc_aux_levels(const hcop_t* h, int64_t* sizes, int32_t max_levels);

/* ---- frequency domain: A = C_nu + i omega M_sigma ------------------------------
 * The complex operator of ComplexMaxwellOperator::Solve
 * (src/formulations/ComplexMaxwell/complex_maxwell_formulation.cpp:171-222:
 * CurlCurlIntegrator in the real part, VectorFEMassIntegrator(omega sigma) in
 * the imaginary part) with permittivity 0 (eddy-current limit).  C_nu is the
 * curl-curl form with the handle's nu alone (no dt), M_sigma the mass form with
 * its sigma; after elimination J = P A P + (I - P).  Structured hex grids.
 * Host vectors use the real-then-imaginary block layout of MFEM's
 * ComplexOperator ([re | im], 2 n_dof doubles); device forms take planar
 * re/im arrays.  omega >= 0.                                                */
hc_status hc_mult_complex(hcop_t* h, double omega, const double* x, double* y);
hc_status hc_mult_complex_device(hcop_t* h, double omega, const double* xr, const double* xi, double* yr,
                                 double* yi);
hc_status hc_mult_complex_device_f32(hcop_t* h, double omega, const float* xr, const float* xi, float* yr,
                                     float* yi);
/* Solve J x = b by COCG (conjugate orthogonal CG: bilinear u^T v products on
 * the complex-symmetric J) with the complex Jacobi preconditioner, in FP64
 * (HC_FP64) or as FP32 inner COCG inside FP64 iterative refinement
 * (HC_MIXED).  Replaces the SuperLU solve of complex_maxwell_formulation.cpp:209-218.
 * precond must be HC_PRECOND_JACOBI; x holds the initial guess.            */
hc_status hc_solve_complex(hcop_t* h, const hc_solve_params* prm, double omega, const double* b, double* x,
                           hc_solve_info* info);
hc_status hc_solve_complex_device(hcop_t* h, const hc_solve_params* prm, double omega, const double* br,
                                  const double* bi, double* xr, double* xi, hc_solve_info* info);
/* Graph-driven form of hc_solve_complex_device: the COCG loop, and for
 * HC_MIXED the refinement loop around it, run inside one CUDA graph whose
 * loops are conditional WHILE nodes with device-side stopping tests (and a
 * hard trip bound), so a solve needs no host round trip per iteration.
 * Enqueues on the handle's stream and returns; hc_graph_solve_info
 * synchronises that stream and reports the solve.  The graph is built on the
 * first call and reused while the arguments (pointers included) stay the same. */
hc_status hc_solve_complex_graph(hcop_t* h, const hc_solve_params* prm, double omega, const double* br,
                                 const double* bi, double* xr, double* xi);
hc_status hc_graph_solve_info(hcop_t* h, hc_solve_info* info);
/* n independent complex solves (batches of uneven problems):
 * every graph is enqueued first, then all are collected, so solves on
 * handles with distinct streams (hc_set_stream) run concurrently.  info[i]
 * gets each solve's report; returns the first non-OK status.               */
hc_status hc_solve_complex_batch(int32_t n, hcop_t* const* hs, const hc_solve_params* prm, const double* omega,
                                 const double* const* br, const double* const* bi, double* const* xr,
                                 double* const* xi, hc_solve_info* info);

/* ---- sources and fields around the solve ----------------------------------- */
/* Points of the q^3 rule the load entry points integrate with (1 <= q <= 8):
 * HC_HEX the tensor Gauss-Legendre rule per element, point kx + q (ky + q kz);
 * HC_TET the collapsed (Duffy) Gauss-Legendre rule, point ic + q (ib + q ia)
 * with barycentrics l1 = u_ia, l2 = u_ib (1 - l1), l3 = u_ic (1 - l1 - l2) on
 * the element's vertices sorted by global id.  xyz: n_elem * q^3 * 3 device
 * doubles, physical coordinates.                                            */
hc_status hc_quad_points_device(hcop_t* h, int q, double* xyz);
/* b = (J, w_i) for a source J the caller supplies (VectorFEDomainLFIntegrator
 * of DivFreeSource::Apply, src/sources/div_free_source.cpp:77-80):
 *   HC_FIELD_ELEM: J holds one vector per element (n_elem * 3), constant there;
 *   HC_FIELD_QUAD: J holds the vector at every point of hc_quad_points_device
 *                  (n_elem * q^3 * 3), integrated with that rule.
 * Device pointers; b is overwritten.                                        */
enum { HC_FIELD_ELEM = 0, HC_FIELD_QUAD = 1 };
hc_status hc_load_field_device(hcop_t* h, int mode, int q, const double* J, double* b);
/* Right-hand side of ScaledCurlVectorGridFunctionAux's projection of
 * H = nu curl A into this Nedelec space, b_i = (nu curl A, w_i), with the
 * handle's per-element nu (MixedVectorCurlIntegrator(nu),
 * src/auxsolvers/scaled_curl_vector_gridfunction_aux.cpp:21-27).  Device.   */
hc_status hc_curl_load_device(hcop_t* h, const double* A, double* b);
/* H = nu curl A projected into this Nedelec space: solves M H = b with the
 * unit-coefficient Nedelec mass M (no essential dofs) by Jacobi PCG to rtol,
 * as ScaledVectorGridFunctionAux::Solve does
 * (src/auxsolvers/scaled_vector_gridfunction_aux.cpp:73-99; the reference
 * registers H = nu curl A this way, src/formulations/HCurl/a_formulation.cpp:78-86).
 * The mass operator is built on the first call and kept by the handle.
 * Device pointers; H holds the initial guess.                               */
hc_status hc_magnetic_field_device(hcop_t* h, const double* A, double* H, double rtol, hc_solve_info* info);
/* B = curl A at npts reference points xi (npts * 3, coordinates in the
 * simplex of the element's vertices sorted by global id: x = v0 + sum_k
 * xi_k (v_k - v0)) of every tet: B is n_elem * npts * 3 physical values
 * (CurlAuxSolver's field, src/auxsolvers/curl_aux.cpp:25-30, sampled
 * pointwise).  Tet meshes; device pointers for A and B, host xi.            */
hc_status hc_tet_curl_points_device(hcop_t* h, const double* A, int npts, const double* xi, double* B);

/* ---- backward-Euler time stepping on device state -------------------------- */
/* b = P (f - C_nu A): one step's right-hand side, the source load f plus
 * WeakCurlCurlKernel's -C_nu A_n (src/kernels/weak_curl_curl_kernel.cpp:27-31),
 * essential rows set to zero (homogeneous A x n = 0, as FormLinearSystem
 * leaves them).  Structured hex grids; device pointers.                    */
hc_status hc_be_rhs_device(hcop_t* h, const double* f, const double* A, double* b);
/* A += dt dA: BackwardEulerSolver's update of the state
 * (src/problem_builders/time_domain_problem_builder.cpp:59-64).  Device.    */
hc_status hc_be_update_device(hcop_t* h, double* A, const double* dA);
/* nsteps backward-Euler steps of TimeDomainEquationSystemProblemOperator::
 * ImplicitSolve (time_domain_equation_system_problem_operator.cpp:31-51):
 * per step b = P (f - C_nu A), dA = 0, solve J dA = b with prm, A += dt dA.
 * f, A, dA, b are device vectors (A is the state, updated in place; dA and
 * b are work vectors that hold the last step's values on return).  info
 * (nsteps entries) receives one report per step taken, status -1 for steps
 * not taken; the loop stops at the first step whose solve is not HC_OK and
 * returns its status.  Structured hex grids.                               */
hc_status hc_be_steps_device(hcop_t* h, const hc_solve_params* prm, int32_t nsteps, const double* f, double* A,
                             double* dA, double* b, hc_solve_info* info);

/* ---- dof correspondence with a caller's numbering (the MFEM shim) ------------
 * The reference passes vectors in MFEM's true-dof numbering of its ND space
 * (EquationSystem::FormLinearSystem / Mult, equation_system.cpp:117-210).
 * Where the caller's local basis on each element is this library's -- MFEM's
 * default ND hex basis read in MFEM's lexicographic element order, and the
 * order-1 (Whitney) tet basis -- the numberings differ by a signed
 * permutation, built here from both sides' element dof lists.  Host code: no
 * device is needed.                                                          */
typedef struct hc_dofmap hc_dofmap_t;
/* This library's dofs of every element of a structured hex grid in the
 * lexicographic local order (x-component dofs (p, p+1, p+1) x fastest, then
 * y, then z): n_elem * 3 p (p+1)^2 entries, elements x fastest.            */
hc_status hc_hex_elem_dofs(int32_t order, int32_t nx, int32_t ny, int32_t nz, int64_t* out);
/* This library's dofs of every tet (order 1: the 6 edges (01,02,03,12,13,23)
 * of the element's vertices sorted by global id; order 2: 20 dofs) and the
 * dof count; numbering as hc_create gives a tet mesh.                       */
hc_status hc_tet_elem_dofs(int32_t order, int64_t n_vert, int64_t n_elem, const int64_t* elem_verts, int64_t* out,
                           int64_t* n_dof);
/* Map from element dof lists: lib_elem_dofs from the calls above,
 * caller_elem_dofs the caller's global dof of the same element and local
 * function (MFEM's encoding: d for +, -1 - d when the element's function is
 * minus the global one).  Fails (HC_EINVAL, reason in hc_dofmap_last_error)
 * unless the correspondence is one to one with one sign per dof.            */
hc_status hc_dofmap_create(int64_t n_dof, int64_t n_elem, int32_t ldofs, const int64_t* lib_elem_dofs,
                           const int32_t* caller_elem_dofs, hc_dofmap_t** out);
/* x_lib = S P x_caller, x_caller = (S P)^T x_lib (host vectors, not aliased) */
hc_status hc_dofmap_to_lib(const hc_dofmap_t* m, const double* x_caller, double* x_lib);
hc_status hc_dofmap_from_lib(const hc_dofmap_t* m, const double* x_lib, double* x_caller);
/* ess_mask (library numbering, n_dof bytes) from the caller's ess_tdof_list
 * (GetEssentialTrueDofs, boundary_conditions.cpp:32-51).                    */
hc_status hc_dofmap_ess_mask(const hc_dofmap_t* m, int64_t n_ess, const int32_t* ess_tdofs, uint8_t* mask);
int64_t hc_dofmap_size(const hc_dofmap_t* m);
hc_status hc_dofmap_last_error(char* buf, size_t n);
void hc_dofmap_destroy(hc_dofmap_t* m);

/* ---- linear solve --------------------------------------------------------- */
/* Solve J x = b for x (x holds the initial guess on entry).  Replaces the
 * HyprePCG solve of HCurlFormulation::ConstructJacobianSolver
 * (hcurl_formulation.cpp:81-85, problem_builder_base.cpp:221-253) for this
 * operator; preconditioner is Jacobi or Chebyshev-Jacobi instead of AMS.
 * Essential rows of b carry the boundary values (MFEM FormLinearSystem).   */
hc_status hc_solve(hcop_t* h, const hc_solve_params* prm, const double* b, double* x,
                   hc_solve_info* info);
hc_status hc_solve_device(hcop_t* h, const hc_solve_params* prm, const double* b, double* x,
                          hc_solve_info* info);
/* Largest eigenvalue estimate of D^-1 J by `steps` Lanczos steps started from
 * v_i = frac(i * 0.6180339887498949) - 1/2.                                */
hc_status hc_lanczos_lmax(hcop_t* h, int steps, double* lmax);
/* z = B r for one preconditioner of the PCG above (device FP64 vectors):
 * HC_PRECOND_JACOBI (B = D^-1) or HC_PRECOND_AUX on hex handles (B = D^-1 +
 * G V G^T, the gradient part of the HypreAMS application, HypreAMS::Mult as
 * the reference's PCG calls it, hcurl_formulation.cpp:69-79).  Lets a caller's
 * own Krylov solver use the library's preconditioner.                      */
hc_status hc_precond_apply_device(hcop_t* h, int32_t precond, const double* r, double* z);

#ifdef __cplusplus
}
#endif
#endif /* HCURL_OP_H */
