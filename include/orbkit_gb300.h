/*
 * orbkit_gb300.h -- C ABI of the GB300 grid-evaluation library (liborbkit_gb300.so).
 *
 * Grid evaluation of contracted Cartesian/spherical Gaussian atomic orbitals and
 * their derivatives, the MO contraction C.AO and the occupation-weighted density
 * and its derivatives, on one GPU (sm_103a).  Every pointer argument named d_* is a
 * device pointer owned by the caller; host arrays are named h_*.  All compute
 * entry points are stream-ordered (they enqueue work on `stream` and return
 * without synchronising) and allocate no memory.  Every function returns an
 * okg_status: 0 on success, a negative code otherwise; okg_last_error() gives
 * a message for the calling thread.
 *
 * Which reference interface each entry point replaces is stated beside it
 * (orbkit file:line).
 */
#ifndef ORBKIT_GB300_H
#define ORBKIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    OKG_OK = 0,
    OKG_ERR_ARG = -1,          /* bad argument, size or pointer */
    OKG_ERR_L = -2,            /* angular momentum above 4, or components of mixed L in one shell */
    OKG_ERR_DRV = -3,          /* derivative code outside 0..9 */
    OKG_ERR_CUDA = -4,         /* CUDA runtime error (launch, copy) */
    OKG_ERR_ALLOC = -5,        /* device or host allocation failed */
    OKG_ERR_TIMEOUT = -6,      /* a bounded device-side wait expired */
    OKG_ERR_UNSUPPORTED = -7,  /* shape outside what the selected kernel supports */
    OKG_ERR_DEVICE = -8        /* no usable sm_103 device */
} okg_status;

typedef void* okg_stream; /* a cudaStream_t; NULL is the legacy default stream */

/* Derivative codes, as orbkit's validate_drv (orbkit/tools.py:225-239):
 * 0 none, 1 x, 2 y, 3 z, 4 xx, 5 yy, 6 zz, 7 xy, 8 xz, 9 yz. */

/* A grid.  regular == 0: vector grid, point i is (x[i], y[i], z[i]).
 * regular == 1: the Nx x Ny x Nz grid spanned by the three coordinate vectors,
 * flattened with x slowest and z fastest (orbkit/cy_grid.pyx:14-30); `offset`
 * is the flattened index of the first point evaluated, npts the number of points. */
typedef struct {
    const double* d_x;
    const double* d_y;
    const double* d_z;
    int64_t npts;
    int64_t offset;
    int32_t nx, ny, nz;
    int32_t regular;
} okg_grid;

typedef struct okg_basis okg_basis;

/* Library status. */
const char* okg_status_string(int status);
const char* okg_last_error(void);
int okg_version(void);

/* Create a basis from orbkit's flattened AO description.
 * Replaces the argument list that orbkit's AOClass getters (orbkit/orbitals.py:336-385)
 * hand to cy_core.aocreator (orbkit/cy_core.pyx:51-78):
 *   h_shell_atom  = ao_spec.get_assign_cont_to_atoms()   (nshell)
 *   h_shell_ncart = ao_spec.get_nlxlylz_per_cont()       (nshell)
 *   h_shell_nprim = ao_spec.get_nprim_per_cont()         (nshell)
 *   h_lxlylz      = ao_spec.get_lxlylz()                 (ncart x 3)
 *   is_normalized = ao_spec.get_normalized()             (orbkit/c_support.c:177-188)
 *   h_renorm      = ao_spec[0]['N'] or NULL              (orbkit/core.py:98-100)
 * Spherical output (orbkit/core.py:135-176): nsph > 0 and, per spherical row r,
 * the components h_sph_cart[h_sph_ptr[r] .. h_sph_ptr[r+1]) (listed Cartesian rows)
 * with coefficients h_sph_coef; rows of one shell must be contiguous.
 * Allocates the device tables on the current device; geometry and primitive
 * exponents/coefficients are set by okg_basis_set_params. */
int okg_basis_create(int natom, int nshell, const int* h_shell_atom, const int* h_shell_ncart,
                     const int* h_shell_nprim, const int* h_lxlylz, int is_normalized, const double* h_renorm,
                     int nsph, const int* h_sph_ptr, const int* h_sph_cart, const double* h_sph_coef,
                     okg_basis** out);
int okg_basis_destroy(okg_basis* basis);
/* Number of Cartesian AOs, output AOs (spherical or Cartesian), shells, primitives, atoms. */
int okg_basis_info(const okg_basis* basis, int* ncart, int* nao, int* nshell, int* nprim, int* natom);

/* Set nuclear positions (d_geo, natom x 3, bohr; orbkit's geo_spec) and primitive
 * exponents/coefficients (d_prim, nprim x 2 [alpha, c]; ao_spec.get_prim_coeffs()).
 * Computes the per-primitive weights c * (2/pi)^(3/4) 2^L alpha^((2L+3)/4)
 * (orbkit/c_support.c:177-188) on `stream`.  Later calls on the same basis must be
 * ordered after this one (same stream, or synchronised). */
int okg_basis_set_params(okg_basis* basis, const double* d_geo, const double* d_prim, okg_stream stream);

/* Column order of the mixed (tensor-core) path: h_order (nshell, host) is a
 * permutation of the shells; whole shells are packed in that order into chunks of
 * 32 columns.  The order changes which K-steps a grid tile's kept shells occupy
 * (the tensor-core work), not the results beyond FP32 summation order.  Only
 * before a mixed plan (okg_mixed_plan_create*, okg_batch_*) or okg_rho_mixed_noalloc
 * used the basis: OKG_ERR_ARG after that, or if h_order is not a permutation.
 * Synchronous (host-to-device copies).  No orbkit counterpart (layout hint). */
int okg_basis_set_mixed_order(okg_basis* basis, const int* h_order);

/* AOs and AO derivatives on a grid, FP64.
 * Replaces cy_core.aocreator + c_lcreator (orbkit/cy_core.pyx:51-78,
 * orbkit/c_grid-based.c:9-79) followed by the 'N' factor and cartesian2spherical
 * (orbkit/core.py:89-102).  h_drv[0..ndrv) are derivative codes; output slot d is
 * d_out[(d * nao + k) * ld + i] for output AO k and point i (AO-major, points
 * contiguous, as ao_list[k, i]).  exact_mixed = 0 evaluates codes 7..9 with orbkit's
 * own formula (orbkit/c_support.c:121-168), 1 with the exact mixed derivative. */
int okg_eval_ao(const okg_basis* basis, const okg_grid* grid, int ndrv, const int* h_drv, int exact_mixed,
                double* d_out, int64_t ld, okg_stream stream);

/* MOs and MO derivatives on a grid, FP64, with the AOs kept on chip.
 * Replaces ao_creator followed by cy_core.mocreator (orbkit/core.py:107-132,
 * orbkit/cy_core.pyx:82-101) for every drv of slice_rho's calc_mo branch
 * (orbkit/core.py:250-263).  d_coeff is C_eff (nmo x ncart, row-major): the MO
 * coefficients in the Cartesian basis (for spherical bases C_sph . T).  Output
 * slot d is d_out[(d * nmo + m) * ld + i]. */
int okg_eval_mo(const okg_basis* basis, const okg_grid* grid, int nmo, const double* d_coeff, int ndrv,
                const int* h_drv, int exact_mixed, double* d_out, int64_t ld, okg_stream stream);

/* Density and density derivatives, FP64, fused AO -> MO -> reduction.
 * Replaces the density part of slice_rho (orbkit/core.py:266-304; also
 * rho_compute_no_slice, orbkit/core.py:808-838):
 *   rho        = sum_m occ_m MO_m^2
 *   drho[d]    = sum_m 2 occ_m dMO_m MO_m                     (codes 1..3)
 *              + sum_m 2 occ_m d_aMO_m d_bMO_m                (codes 4..9, two-letter selectors)
 * d_rho[i], d_drho[d * ld + i]; d_drho may be NULL when ndrv == 0.
 * d_mo_norm (nmo, or NULL) receives += sum_i MO_m(i)^2 (atomic, order not fixed). */
int okg_rho(const okg_basis* basis, const okg_grid* grid, int nmo, const double* d_coeff, const double* d_occ,
            int ndrv, const int* h_drv, int exact_mixed, double* d_rho, double* d_drho, int64_t ld,
            double* d_mo_norm, okg_stream stream);

/* ------------------------------------------------ operations on given grids
 * FP64 operations on AO / MO values the caller already holds on the device, every
 * array row-major (row, point) with points contiguous and its own leading dimension
 * (ld >= npts), as orbkit's ao_list[k, i] / mo_list[m, i]. */
/* MO = C . AO: d_out[m * ld_out + i] = sum_k d_coeff[m * nao + k] d_ao[k * ld_ao + i]
 * (FMA accumulation).  Replaces cy_core.mocreator (orbkit/cy_core.pyx:82-101) behind
 * core.mo_creator (orbkit/core.py:107-132). */
int okg_mo_from_ao(int nmo, int nao, const double* d_coeff, const double* d_ao, int64_t ld_ao, int64_t npts,
                   double* d_out, int64_t ld_out, okg_stream stream);
/* Spherical rows from Cartesian rows: d_out[r * ld_out + i] = sum over t in
 * [d_ptr[r], d_ptr[r+1]) of d_coef[t] d_in[d_cart[t] * ld_in + i], terms added in
 * order with one rounding per product and per sum (orbkit's numpy arithmetic, bit for
 * bit).  d_cart entries must lie in [0, ncart) (others give NaN).  Replaces
 * core.cartesian2spherical (orbkit/core.py:135-176); the CSR arrays are those of
 * okg_basis_create's spherical transform (coefficient x global factor). */
int okg_cart2sph(int nsph, int ncart, const int* d_ptr, const int* d_cart, const double* d_coef, const double* d_in,
                 int64_t ld_in, int64_t npts, double* d_out, int64_t ld_out, okg_stream stream);
/* MO products of calc_mo_matrix (orbkit/core.py:935-937):
 * d_out[((d * na + n) * nb + m) * ld_out + i] = d_bra[n * ld_bra + i] * d_ket[(d * nb + m) * ld_ket + i]
 * (one rounded multiply: orbkit's values bit for bit). */
int okg_mo_products(int ndrv, int na, int nb, const double* d_bra, int64_t ld_bra, const double* d_ket,
                    int64_t ld_ket, int64_t npts, double* d_out, int64_t ld_out, okg_stream stream);
/* Transition flux densities of extras.calc_jmo (orbkit/extras.py:441-492) for MO
 * pairs (i, j) = (d_pairs[2q], d_pairs[2q+1]) in [0, nmo) (others give NaN):
 * d_out[(d * npair + q) * ld_out + p] = -0.5 (bra_i ket_{d,j} - bra_j ket_{d,i}), with
 * bra_i = d_bra[i * ld_bra + p] and ket_{d,j} = d_ket[(d * nmo + j) * ld_ket + p]
 * (orbkit's numpy rounding, bit for bit). */
int okg_mo_pair_flux(int ndrv, int nmo, int npair, const int* d_pairs, const double* d_bra, int64_t ld_bra,
                     const double* d_ket, int64_t ld_ket, int64_t npts, double* d_out, int64_t ld_out,
                     okg_stream stream);

/* ---------------------------------------------------------------- mixed path
 * rho and grad rho with the C.AO contraction on the tensor cores (tcgen05, BF16
 * operands split three ways, FP32 accumulation), exponent arguments and the final
 * density accumulation in FP64.  Same quantities as okg_rho with codes {1,2,3}
 * (orbkit/core.py:266-300), within the error stated by the tests.
 * A plan holds the tensor-core operand form of the MO coefficients. */
typedef struct okg_mixed_plan okg_mixed_plan;
/* Allocates the plan's device buffer (split coefficients, occupations, status word).
 * OKG_ERR_UNSUPPORTED for bases beyond the kernel's shared-memory tables: more than
 * 2048 shells, 192 column chunks or 31 primitives in a shell (the FP64 path has no
 * such limits). */
int okg_mixed_plan_create(const okg_basis* basis, int nmo, okg_mixed_plan** out);
/* Same with the MMA's N tile (MO columns per pass over the AO chunks) limited to
 * n_max (16, 32, 48 or 64; okg_mixed_plan_create uses 64): a tile shape for the
 * autotuner -- fewer columns per pass, more passes. */
int okg_mixed_plan_create_tiled(const okg_basis* basis, int nmo, int n_max, okg_mixed_plan** out);
int okg_mixed_plan_destroy(okg_mixed_plan* plan);
/* AO-generation threads per CTA of the plan's launches: 256, 384 or 512, one grid
 * point each (2, 3 or 4 threads share the AO generation of each of the tile's 128
 * points); one more warp issues the tensor-core work. */
int okg_mixed_plan_set_threads(okg_mixed_plan* plan, int threads);
/* The same with the grid points per generation thread: (256, 1), (384, 1), (512, 1),
 * (256, 2) or (384, 2).  With 2 points a thread generates two adjacent points of the
 * tile (packed conversions and stores); default (384, 1). */
int okg_mixed_plan_set_generation(okg_mixed_plan* plan, int threads, int points_per_thread);
/* Split C_eff (nmo x ncart, FP64, device) into the BF16 operand tiles; copy occ (nmo). */
int okg_mixed_set_coeffs(okg_mixed_plan* plan, const double* d_coeff, const double* d_occ, okg_stream stream);
/* d_rho[i]; d_grad[c * ld + i] for c = x, y, z when want_grad.  Every point is
 * evaluated by the tensor-core kernel, the cusp region near nuclei included: the
 * Python layer (orbkit_gb300.mixed) recomputes the points near nuclei with okg_rho. */
int okg_rho_mixed(okg_mixed_plan* plan, const okg_grid* grid, int want_grad, double* d_rho, double* d_grad,
                  int64_t ld, okg_stream stream);
/* Synchronising check of the plan's device status word (bounded tensor-core waits):
 * OKG_ERR_TIMEOUT if a wait expired since the last check (the word is then cleared). */
int okg_mixed_status(okg_mixed_plan* plan, int* device_status);
/* Polls per bounded device wait of the plan's launches (default 2^24, >= 1).  When a
 * wait expires the kernel raises the status word, stops issuing tensor-core work,
 * waits for its own bulk copies and MMAs in flight, frees its tensor memory and
 * returns (the outputs are then incomplete); the next launch starts afresh.  A small
 * limit makes a wait expire on purpose, which is how the timeout path is tested. */
int okg_mixed_plan_set_wait_limit(okg_mixed_plan* plan, long long polls);
/* FP64 cusp region inside the tensor-core kernel (no counterpart in orbkit, which is
 * FP64 everywhere): d_near (device, one int16 per point of the grids later passed with
 * this plan -- the call's point index -- or NULL to switch off) names the atom within
 * whose cusp radius the point lies, or -1.  In every 128-point tile that holds such a
 * point, the primitives with alpha > alpha_c of the atoms named there are left out of
 * the BF16 operand; the epilogue evaluates them in FP64 at each point of the tile (exp,
 * radial sums, polynomials; those below e^-50 at the point dropped), contracts them with
 * C_eff in FP64 and forms the point's density products in FP64.  More than 8 such atoms
 * in one tile is reported by okg_mixed_status / okg_batch_status as OKG_ERR_UNSUPPORTED.  The plan keeps the pointer (the caller keeps the
 * array alive); a batch takes the setting of each molecule's plan at okg_batch_create. */
int okg_mixed_plan_set_cusp(okg_mixed_plan* plan, const int16_t* d_near, double alpha_c);

/* ------------------------------------------------------------------- batches
 * Many molecules with uneven point sets (e.g. atom-centred grids) in one
 * persistent launch of the mixed kernel: no counterpart in orbkit, which evaluates
 * one molecule per call (orbkit/core.py:314); each molecule's result is what
 * okg_rho_mixed gives for it.  The batch holds one (plan, grid, outputs) entry per
 * molecule; tiles of 128 points are numbered across molecules in the given order
 * and handed out to one CTA per SM through a device counter.  okg_batch_run is a
 * counter reset plus one kernel launch on `stream` and can be captured in a CUDA
 * graph.  okg_batch_set_schedule sets the tiles taken per counter increment, the
 * number of CTAs and the threads per CTA (the autotuner's knobs). */
typedef struct okg_batch okg_batch;
int okg_batch_create(int nmol, okg_mixed_plan* const* plans, const okg_grid* grids, double* const* d_rho,
                     double* const* d_grad, const int64_t* ld, int want_grad, okg_batch** out);
int okg_batch_destroy(okg_batch* batch);
int okg_batch_set_schedule(okg_batch* batch, int tiles_per_grab, int ctas, int threads);
/* Generation threads and grid points per generation thread as for
 * okg_mixed_plan_set_generation (after okg_batch_set_schedule, which sets one point). */
int okg_batch_set_generation(okg_batch* batch, int threads, int points_per_thread);
int okg_batch_tiles(const okg_batch* batch, long long* total_tiles);
int okg_batch_run(okg_batch* batch, okg_stream stream);
int okg_batch_status(okg_batch* batch, int* device_status);

/* ------------------------------------------------------------------- adjoint
 * Gradients of a loss L(rho, grad rho) with respect to the MO coefficients, the
 * primitive exponents and contraction coefficients, and the nuclear coordinates,
 * given the cotangents d_g_rho = dL/drho (npts) and d_g_grad = dL/d(grad rho)
 * (3 x ld, or NULL).  Differentiates the forward of okg_rho with codes {1,2,3}
 * (orbkit/core.py:266-300; AO math of orbkit/c_grid-based.c:9-79 and
 * orbkit/c_support.c:28-188); AO tiles are recomputed, not stored.
 * Outputs (overwritten): d_dcoeff (nmo x ncart, w.r.t. C_eff), d_dprim (nprim x 2:
 * d/dalpha, d/dc in ao_spec.get_prim_coeffs() order), d_dgeo (natom x 3).
 * precision: 64 or 32 (arithmetic of the backward).  Any nmo: above 48 MOs the AO
 * tiles of the MO pass are recomputed per block of 48 MOs.  d_work is caller
 * memory of at least okg_rho_backward_workspace bytes (per-CTA partial sums,
 * reduced in a fixed order: results are deterministic). */
int okg_rho_backward_workspace(const okg_basis* basis, const okg_grid* grid, int nmo, int precision, size_t* bytes);
int okg_rho_backward(const okg_basis* basis, const okg_grid* grid, int nmo, const double* d_coeff,
                     const double* d_occ, const double* d_g_rho, const double* d_g_grad, int64_t ld, int precision,
                     double* d_dcoeff, double* d_dprim, double* d_dgeo, void* d_work, size_t work_bytes,
                     okg_stream stream);

/* Allocation-free variant of okg_rho_mixed; no counterpart in orbkit.
 * For callers that cannot allocate device memory where they evaluate the density
 * (a framework that owns all device memory through its own pool, or a loop that
 * cannot take cudaMalloc's implicit device synchronisation).  The MO coefficients
 * d_coeff (C_eff, nmo x ncart) and occupations d_occ are split into a 2 MiB
 * file-scope device array on every call instead of a plan's buffer; larger
 * (basis, nmo) combinations return OKG_ERR_UNSUPPORTED.  The first call on a device
 * looks up the array and sets up the kernel (make it before any stream capture);
 * the looked-up address is kept for the process, so do not use this entry point
 * across a cudaDeviceReset.  Calls that overlap on the GPU race on the shared array.
 * d_status (required, a device int) is cleared by the call and set to 1 by the
 * kernel if a tensor-core wait expired (the outputs are then incomplete).  As with
 * okg_rho_mixed, every point -- the cusp region near nuclei included -- comes from
 * the tensor-core kernel (no FP64 recomputation at this level). */
int okg_rho_mixed_noalloc(const okg_basis* basis, const okg_grid* grid, int nmo, const double* d_coeff,
                          const double* d_occ, int want_grad, double* d_rho, double* d_grad, int64_t ld,
                          int* d_status, okg_stream stream);

/* ------------------------------------------------------------------- detCI
 * CI (transition) densities and flux densities on a grid from MO grids d_mo
 * (nmo x ld, points contiguous: orbkit's molist) and, for the fluxes, their x, y, z
 * derivatives d_drv (3 x nmo x ld: orbkit's molistdrv).  The terms come from
 * orbkit's determinant comparison (orbkit/detci/occ_check.py): "zero" terms
 * (coefficient d_zcoef[t], orbital d_zidx[t]) and single-excitation terms
 * (coefficient d_scoef[t], orbitals d_spair[2t], d_spair[2t+1]), all on the device.
 * Terms are summed in the given order with orbkit's rounding of every product and
 * sum (no FMA contraction). */
/* rho[p] = sum_t zc[t] MO_zi[t](p)^2 + sum_t sc[t] MO_a(p) MO_b(p):
 * replaces orbkit/detci/cy_ci.pyx:70-96 (get_rho) behind detci.ci_core.rho. */
int okg_ci_rho(int64_t npts, const double* d_mo, int64_t ld, int nz, const double* d_zcoef, const int* d_zidx,
               int ns, const double* d_scoef, const int* d_spair, double* d_rho, okg_stream stream);
/* j[d*npts + p] = -sum_t 0.5 sc[t] (MO_a dMO_b - MO_b dMO_a), d = x, y, z:
 * replaces orbkit/detci/cy_ci.pyx:152-178 (get_jab) behind detci.ci_core.jab. */
int okg_ci_jab(int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo, int ns,
               const double* d_scoef, const int* d_spair, double* d_j, okg_stream stream);
/* j[d*npts + p] = sum_t sc[t] MO_a dMO_b: replaces orbkit/detci/cy_ci.pyx:203-229
 * (get_a_nabla_b) behind detci.ci_core.a_nabla_b. */
int okg_ci_a_nabla_b(int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo, int ns,
                     const double* d_scoef, const int* d_spair, double* d_j, okg_stream stream);

/* The same sums as quadratic forms (no counterpart in orbkit; a faster evaluation
 * of ci_core.rho / jab / a_nabla_b, orbkit/detci/ci_core.py:84-267): the host folds
 * the terms into NMO x NMO matrices and a point costs NMO^2 FMAs whatever the
 * number of terms.  d_qt holds nmo rows of ldq = nmo rounded up to a multiple of 16
 * doubles (zero padded, 16-byte aligned).
 * rho[p] = sum_b MO_b(p) sum_{a <= b} qt[b*ldq + a] MO_a(p)   (qt lower triangular:
 *          the symmetrised density matrix, M_ab + M_ba off the diagonal) */
int okg_ci_rho_matrix(int64_t npts, const double* d_mo, int64_t ld, int nmo, const double* d_qt, double* d_rho,
                      okg_stream stream);
/* j[d*npts + p] = scale sum_b dMO_b(p) sum_a qt[b*ldq + a] MO_a(p), d = x, y, z
 * (jab: qt = C^T - C, scale = -1/2; a_nabla_b: qt = C^T, scale = 1, with C_ab the
 * summed coefficients of the single-excitation terms (a, b)). */
int okg_ci_flux_matrix(int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo,
                       const double* d_qt, double scale, double* d_j, okg_stream stream);

/* ------------------------------------------------------------ AO overlap
 * Analytic overlap of contracted Cartesian Gaussians, FP64:
 * replaces cy_overlap.aooverlap (orbkit/cy_overlap.pyx:78-163, with get_overlap of
 * orbkit/c_non-grid-based.c:9-52) and the 'N' factor / cartesian2spherical_aoom steps
 * of get_ao_overlap (orbkit/analytical_integrals.py:37-182).
 * The plan takes the arrays of okg_basis_create plus the primitives (h_prim,
 * nprim x 2 [alpha, c]; ao_spec.get_prim_coeffs()) on the host; per (listed row,
 * primitive) norms ao_norm (orbkit/c_support.c:177-188) are computed once from the
 * bra exponents h_lxlylz, as orbkit does for both bra and ket.  The plan allocates its
 * device tables, an ncart x ncart workspace and, when it takes at most 2 GiB, an
 * nprim x nprim x 48-byte table of primitive-pair quantities that every okg_ao_overlap
 * call refills for its geometries. */
typedef struct okg_overlap_plan okg_overlap_plan;
int okg_overlap_plan_create(int natom, int nshell, const int* h_shell_atom, const int* h_shell_ncart,
                            const int* h_shell_nprim, const int* h_lxlylz, int is_normalized, const double* h_prim,
                            const double* h_renorm, int nsph, const int* h_sph_ptr, const int* h_sph_cart,
                            const double* h_sph_coef, okg_overlap_plan** out);
int okg_overlap_plan_destroy(okg_overlap_plan* plan);
/* Listed Cartesian rows and output rows (spherical if the plan has a transform). */
int okg_overlap_plan_info(const okg_overlap_plan* plan, int* ncart, int* nao);
/* Ket exponents (ncart x 3; get_ao_overlap's lxlylz_b), NULL = the bra's.  Synchronous. */
int okg_overlap_plan_set_ket(okg_overlap_plan* plan, const int* h_lxlylz_b);
/* d_out[I * ld + J] = <bra I at d_geo_a | d^drv ket J at d_geo_b> (natom x 3 each, on the
 * device); drv 0 none, 1..3 d/dx, d/dy, d/dz of the ket.  raw = 1 returns the Cartesian
 * matrix of cy_overlap.aooverlap; raw = 0 applies the 'N' factor and the spherical
 * transform as get_ao_overlap does (nao x nao). */
int okg_ao_overlap(okg_overlap_plan* plan, const double* d_geo_a, const double* d_geo_b, int drv, int raw,
                   double* d_out, int64_t ld, okg_stream stream);

/* Diagnostic (no counterpart in orbkit): measured FP64 FMA rate of the current device
 * in FMA/s, from a kernel of independent FMA chains (synchronising; allocates). */
int okg_diag_fp64_fma_rate(long long iters, double* fma_per_s);

#ifdef __cplusplus
}
#endif
#endif /* ORBKIT_GB300_H */
