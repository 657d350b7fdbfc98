/*
 * hcurl_oracle.h -- FP64 CPU oracle for the H(curl) curl-curl + mass hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  The
 * product (hephaestus_gb300) never links or calls it.
 *
 * It is an independent restatement of what the reference computes on this
 * path.  The reference delegates all arithmetic to MFEM (fork
 * Heinrich-BR/mfem@SubmeshBoundary, no commit pinned, see
 * docker/hephaestus-deps/Dockerfile:115-141) and hypre (via PETSc 3.19.3);
 * neither is vendored, so the algorithms below are restated from the
 * published mathematics, anchored on the reference's call sites:
 *
 *  - bilinear form a1(u,u') = (beta u,u') + (alpha dt curl u, curl u')
 *      src/formulations/HCurl/hcurl_formulation.cpp:1-38,130-157
 *      src/kernels/curl_curl_kernel.cpp:21-24   (CurlCurlIntegrator)
 *      src/kernels/vector_fe_mass_kernel.cpp:21-24 (VectorFEMassIntegrator)
 *  - essential tangential dofs + elimination with unit diagonal
 *      src/boundary_conditions/boundary_conditions.cpp:32-51
 *      src/equation_systems/equation_system.cpp:117-198
 *  - PCG with Jacobi (HypreDiagScale) preconditioning
 *      src/solvers/hephaestus_solvers.hpp:34-57
 *  - right-hand side (J, w_i)       src/sources/div_free_source.cpp:72-114
 *  - WeakCurlCurl RHS term -C_nu A_n src/kernels/weak_curl_curl_kernel.cpp:27-31
 *
 * Nedelec (first kind) bases: on hexes the tensor product of a closed
 * (Gauss-Lobatto nodal, degree p) and an open (Gauss-Legendre nodal, degree
 * p-1) 1-D basis; on tets the hierarchical Whitney-type basis
 * lambda_a (lambda_b grad lambda_c - lambda_c grad lambda_b) with vertices
 * ordered by global index.  Since these differ from MFEM's, per-dof values
 * compare to the reference only through basis-invariant quantities (MMS
 * errors and rates, energies); the known-answer pin is the reference's MMS
 * convergence test test/integration/test_aform_source.cpp:130-209.
 */
#ifndef HCURL_ORACLE_H
#define HCURL_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- problem construction ---------------------------------------------- */
/* Structured nx*ny*nz hex grid, Nedelec order p (1..4).  verts holds
 * (nx+1)(ny+1)(nz+1) points, x fastest; NULL means the unit cube.         */
void*   orc_hex_new(int nx, int ny, int nz, int p, const double* verts);
/* Tet mesh: nv vertices (xyz), ne tets (4 vertex ids each), order p (1,2). */
void*   orc_tet_new(int64_t nv, const double* verts, int64_t ne, const int64_t* tets, int p);
void    orc_free(void* h);

int64_t orc_ndof(void* h);
int64_t orc_nelem(void* h);
int     orc_ldof(void* h);
void    orc_elem_dofs(void* h, int64_t* out);           /* ne * ldof      */
int64_t orc_tet_nedges(void* h);
int64_t orc_tet_nfaces(void* h);

/* ---- coefficients and assembly ------------------------------------------ */
/* Per-element constants: alpha multiplies curl-curl (dt*nu in the A-form),
 * beta multiplies the mass (sigma).  beta may be NULL (magnetostatic).     */
void    orc_set_coef(void* h, const double* alpha, const double* beta);
/* Manufactured-solution coefficients of test_aform_source.cpp:32-57:
 * alpha(x) = dt * (1 + s cos(pi x) cos(pi y)), beta = sigma.                */
void    orc_set_coef_mms(void* h, double dt, double var_scale, double sigma);
/* Points per direction of the element-matrix rules for the curl-curl and
 * mass terms (0 = default rule, exact for affine elements and constant
 * coefficients).                                                           */
void    orc_set_quad(void* h, int q_curl, int q_mass);
int     orc_assemble(void* h, int nthreads);
int64_t orc_nnz(void* h);
void    orc_csr(void* h, int64_t* rowptr, int64_t* col, double* val);
void    orc_element_matrix(void* h, int64_t e, double* out);   /* ldof^2 */

/* ---- essential dofs, masked (eliminated) operator ----------------------- */
/* Hex faces carry attributes 1..6 = x-,x+,y-,y+,z-,z+; bit (a-1) of
 * attr_bits selects attribute a.                                            */
void    orc_hex_ess_mask(void* h, int attr_bits, uint8_t* mask);
/* Tet: boundary triangles (3 vertex ids) with attributes.                   */
void    orc_tet_ess_mask(void* h, int64_t nb, const int64_t* tris, const int* attr,
                         int attr_bits, uint8_t* mask);
void    orc_set_ess(void* h, const uint8_t* mask);

void    orc_apply(void* h, const double* x, double* y, int nthreads);        /* K x      */
void    orc_apply_masked(void* h, const double* x, double* y, int nthreads); /* PKPx+(I-P)x */
void    orc_diag_masked(void* h, double* d);
/* Eliminated operator stored as hypre holds it (ess rows/cols removed, unit
 * diagonal, 32-bit columns); returns its nnz.  Used for the CPU baseline.  */
int64_t orc_build_eliminated(void* h);
void    orc_spmv_eliminated(void* h, const double* x, double* y, int nthreads);
/* Curl-curl part alone (alpha only) -- WeakCurlCurlKernel's C_nu action.   */
void    orc_apply_curlcurl(void* h, const double* x, double* y);

/* ---- solvers ------------------------------------------------------------ */
/* precond: 0 none, 1 Jacobi, 2 Chebyshev-Jacobi of degree cheb_degree on
 * [lmax/cheb_ratio, lmax]; lmax <= 0 means estimate it by Lanczos.
 * Returns 0 converged, 4 not converged, 5 breakdown.                        */
int     orc_pcg(void* h, const double* b, double* x, int precond, int cheb_degree,
                double cheb_lmax, double cheb_ratio, double rtol, double atol, int maxit,
                int nthreads, int* iters, double* relres);
double  orc_lanczos_lmax(void* h, int steps, int nthreads);
/* y = Chebyshev-Jacobi preconditioner applied to r. */
void    orc_cheb_apply(void* h, int degree, double lmax, double ratio, const double* r,
                       double* z, int nthreads);

/* ---- right-hand sides, errors, curl ------------------------------------- */
/* Loop coil J = I0 (-(y-yc), x-xc, 0) in r0<=r<=r1, z0<=z<=z1.  Gauss rule
 * with q points per direction per hex (or q^3 collapsed points per tet).    */
void    orc_load_coil(void* h, double I0, double xc, double yc, double r0, double r1, double z0,
                      double z1, int q, double* b);
/* b_i = (J, w_i) for J constant per element (ne x 3), and for the affine
 * J(x) = a + B x (B row-major 3x3); the same q-point rules as orc_load_coil. */
void    orc_load_elem_field(void* h, const double* J, int q, double* b);
void    orc_load_affine(void* h, const double* a, const double* B, int q, double* b);
/* b_i = (nu curl A, w_i), nu constant per element (ne values).             */
void    orc_curl_load(void* h, const double* nu, const double* A, int q, double* b);
/* Source of test_aform_source.cpp:39-49 at time t.                          */
void    orc_load_mms(void* h, double t, double var_scale, int q, double* b);
/* L2 norm of (A_h - A_exact(t)), A_exact = t sin(pi y) sin(pi z) e_x.     */
double  orc_l2err_mms(void* h, const double* A, double t, int q);
/* Physical field and curl of the dof vector at reference point xi of element e. */
void    orc_eval(void* h, const double* A, int64_t e, const double* xi, double* val, double* curl);

#ifdef __cplusplus
}
#endif
#endif
