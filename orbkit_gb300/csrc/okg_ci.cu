// CI (transition) densities and flux densities on a grid from MO grids: the grid
// loops of orbkit's detCI module (orbkit/detci/cy_ci.pyx:70-96 get_rho,
// :152-178 get_jab, :203-229 get_a_nabla_b; drivers orbkit/detci/ci_core.py:84-267).
//
// Inputs are the MO grids (nmo x ld, points contiguous, as orbkit's molist) and the
// determinant-comparison terms of orbkit/detci/occ_check.py: "zero" terms
// (coefficient, orbital) contribute c MO_s^2, "single" terms (coefficient, orbital
// pair a, b) contribute c MO_a MO_b.  One thread per grid point walks the terms in
// the given order with each product and sum rounded as orbkit writes it (no FMA
// contraction), so for the same MO grids the results are orbkit's to the bit.
// Term tables are read by every thread of a warp at the same address (broadcast
// through L1); MO values are read coalesced.
#include "okg_internal.cuh"

namespace okg {

__global__ void ci_rho_kernel(long long npts, const double* __restrict__ mo, long long ld, int nz,
                              const double* __restrict__ zc, const int* __restrict__ zi, int ns,
                              const double* __restrict__ sc, const int* __restrict__ sp, double* __restrict__ rho)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    double r = 0.0;
    for (int t = 0; t < nz; ++t) {
        const double m = mo[(long long)__ldg(zi + t) * ld + p];
        r = __dadd_rn(r, __dmul_rn(__dmul_rn(__ldg(zc + t), m), m));
    }
    for (int t = 0; t < ns; ++t) {
        const double ma = mo[(long long)__ldg(sp + 2 * t) * ld + p];
        const double mb = mo[(long long)__ldg(sp + 2 * t + 1) * ld + p];
        r = __dadd_rn(r, __dmul_rn(__dmul_rn(__ldg(sc + t), ma), mb));
    }
    rho[p] = r;
}

// ANTISYM: j_d -= 0.5 (c (MO_a dMO_b - MO_b dMO_a))  (get_jab)
// else:    j_d += c (MO_a dMO_b)                       (get_a_nabla_b)
template <bool ANTISYM>
__global__ void ci_flux_kernel(long long npts, const double* __restrict__ mo, const double* __restrict__ drv,
                               long long ld, int nmo, int ns, const double* __restrict__ sc,
                               const int* __restrict__ sp, double* __restrict__ j)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const long long dstride = (long long)nmo * ld;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < ns; ++t) {
        const int a = __ldg(sp + 2 * t), b = __ldg(sp + 2 * t + 1);
        const double c = __ldg(sc + t);
        const double ma = mo[(long long)a * ld + p];
        const double mb = mo[(long long)b * ld + p];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double db = drv[d * dstride + (long long)b * ld + p];
            if (ANTISYM) {
                const double da = drv[d * dstride + (long long)a * ld + p];
                const double t2 = __dmul_rn(0.5, __dmul_rn(c, __dsub_rn(__dmul_rn(ma, db), __dmul_rn(mb, da))));
                acc[d] = __dsub_rn(acc[d], t2);
            } else {
                acc[d] = __dadd_rn(acc[d], __dmul_rn(c, __dmul_rn(ma, db)));
            }
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) j[(long long)d * npts + p] = acc[d];
}

// Quadratic-form evaluation of the same sums.  The terms collapse into NMO x NMO
// coefficient matrices (host side): rho = sum_ab M_ab MO_a MO_b and
// j_d = scale sum_ab Q_ab MO_a dMO_b, so a point costs NMO^2 FMAs instead of work
// proportional to the number of terms.  Each thread owns one point and walks the
// bra orbitals in chunks of CI_CH held in registers; per ket orbital b it forms
// t_b = sum_{a in chunk} Q^T[b][a] MO_a (coefficients read as broadcasts through
// L1) and adds t_b MO_b (rho) or t_b dMO_b for the three directions (flux), so the
// flux shares one matrix-vector product between x, y and z.  For rho the matrix is
// symmetrised and only a <= b is visited (lower triangle of Q^T, zero above).
// FP64 FMAs; the sum order differs from orbkit's term order.
#define CI_CH 16

template <bool FLUX>
__global__ void __launch_bounds__(128) ci_quad_kernel(long long npts, const double* __restrict__ mo,
                                                      const double* __restrict__ drv, long long ld, int nmo,
                                                      const double* __restrict__ qt, double scale,
                                                      double* __restrict__ out)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const long long dstride = (long long)nmo * ld;
    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
    for (int a0 = 0; a0 < nmo; a0 += CI_CH) {
        double pa[CI_CH];
#pragma unroll
        for (int i = 0; i < CI_CH; ++i) pa[i] = (a0 + i < nmo) ? mo[(long long)(a0 + i) * ld + p] : 0.0;
        // rho: rows b < a0 of the lower-triangular Q^T hold zeros for this chunk
        for (int b = FLUX ? 0 : a0; b < nmo; ++b) {
            const double2* q = reinterpret_cast<const double2*>(qt + (long long)b * ((nmo + CI_CH - 1) / CI_CH * CI_CH) + a0);
            double t = 0.0;
#pragma unroll
            for (int i = 0; i < CI_CH / 2; ++i) {
                const double2 c = __ldg(q + i);
                t = fma(c.x, pa[2 * i], t);
                t = fma(c.y, pa[2 * i + 1], t);
            }
            if (FLUX) {
                acc0 = fma(t, drv[(long long)b * ld + p], acc0);
                acc1 = fma(t, drv[dstride + (long long)b * ld + p], acc1);
                acc2 = fma(t, drv[2 * dstride + (long long)b * ld + p], acc2);
            } else {
                acc0 = fma(t, mo[(long long)b * ld + p], acc0);
            }
        }
    }
    if (FLUX) {
        out[p] = scale * acc0;
        out[npts + p] = scale * acc1;
        out[2 * npts + p] = scale * acc2;
    } else {
        out[p] = scale * acc0;
    }
}

}  // namespace okg

using namespace okg;

static int ci_check_terms(int n, const double* c, const int* idx, const char* what)
{
    if (n < 0 || (n > 0 && (!c || !idx))) return set_error(OKG_ERR_ARG, what);
    return OKG_OK;
}

extern "C" int okg_ci_rho(int64_t npts, const double* d_mo, int64_t ld, int nz, const double* d_zcoef,
                          const int* d_zidx, int ns, const double* d_scoef, const int* d_spair, double* d_rho,
                          okg_stream stream)
{
    if (npts < 0 || !d_rho || (npts > 0 && !d_mo) || ld < npts)
        return set_error(OKG_ERR_ARG, "okg_ci_rho: NULL MO grid / output, npts < 0 or ld < npts");
    int st = ci_check_terms(nz, d_zcoef, d_zidx, "okg_ci_rho: zero-term table NULL or nz < 0");
    if (st) return st;
    if ((st = ci_check_terms(ns, d_scoef, d_spair, "okg_ci_rho: single-term table NULL or ns < 0"))) return st;
    if (npts == 0) return OKG_OK;
    const unsigned nblk = (unsigned)((npts + 127) / 128);
    ci_rho_kernel<<<nblk, 128, 0, (cudaStream_t)stream>>>(npts, d_mo, ld, nz, d_zcoef, d_zidx, ns, d_scoef, d_spair,
                                                          d_rho);
    return cuda_status(cudaGetLastError(), "okg_ci_rho launch");
}

static int ci_flux(bool antisym, int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo, int ns,
                   const double* d_scoef, const int* d_spair, double* d_j, cudaStream_t st, const char* name)
{
    if (npts < 0 || !d_j || (npts > 0 && (!d_mo || !d_drv)) || ld < npts || nmo <= 0)
        return set_error(OKG_ERR_ARG, name);
    int s = ci_check_terms(ns, d_scoef, d_spair, name);
    if (s) return s;
    if (npts == 0) return OKG_OK;
    const unsigned nblk = (unsigned)((npts + 127) / 128);
    if (antisym)
        ci_flux_kernel<true><<<nblk, 128, 0, st>>>(npts, d_mo, d_drv, ld, nmo, ns, d_scoef, d_spair, d_j);
    else
        ci_flux_kernel<false><<<nblk, 128, 0, st>>>(npts, d_mo, d_drv, ld, nmo, ns, d_scoef, d_spair, d_j);
    return cuda_status(cudaGetLastError(), name);
}

extern "C" int okg_ci_jab(int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo, int ns,
                          const double* d_scoef, const int* d_spair, double* d_j, okg_stream stream)
{
    return ci_flux(true, npts, d_mo, d_drv, ld, nmo, ns, d_scoef, d_spair, d_j, (cudaStream_t)stream,
                   "okg_ci_jab: bad argument (NULL pointer, npts < 0, ld < npts, nmo <= 0 or ns < 0)");
}

extern "C" int okg_ci_a_nabla_b(int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo, int ns,
                                const double* d_scoef, const int* d_spair, double* d_j, okg_stream stream)
{
    return ci_flux(false, npts, d_mo, d_drv, ld, nmo, ns, d_scoef, d_spair, d_j, (cudaStream_t)stream,
                   "okg_ci_a_nabla_b: bad argument (NULL pointer, npts < 0, ld < npts, nmo <= 0 or ns < 0)");
}

// Q^T is nmo rows of ldq = nmo rounded up to a multiple of 16 doubles (zero padded;
// 16-byte aligned rows).
extern "C" int okg_ci_rho_matrix(int64_t npts, const double* d_mo, int64_t ld, int nmo, const double* d_qt,
                                 double* d_rho, okg_stream stream)
{
    if (npts < 0 || !d_rho || (npts > 0 && (!d_mo || !d_qt)) || ld < npts || nmo <= 0)
        return set_error(OKG_ERR_ARG, "okg_ci_rho_matrix: bad argument (NULL pointer, npts < 0, ld < npts, nmo <= 0)");
    if (((uintptr_t)d_qt & 15) != 0) return set_error(OKG_ERR_ARG, "okg_ci_rho_matrix: d_qt not 16-byte aligned");
    if (npts == 0) return OKG_OK;
    const unsigned nblk = (unsigned)((npts + 127) / 128);
    ci_quad_kernel<false><<<nblk, 128, 0, (cudaStream_t)stream>>>(npts, d_mo, nullptr, ld, nmo, d_qt, 1.0, d_rho);
    return cuda_status(cudaGetLastError(), "okg_ci_rho_matrix launch");
}

extern "C" int okg_ci_flux_matrix(int64_t npts, const double* d_mo, const double* d_drv, int64_t ld, int nmo,
                                  const double* d_qt, double scale, double* d_j, okg_stream stream)
{
    if (npts < 0 || !d_j || (npts > 0 && (!d_mo || !d_drv || !d_qt)) || ld < npts || nmo <= 0)
        return set_error(OKG_ERR_ARG, "okg_ci_flux_matrix: bad argument (NULL pointer, npts < 0, ld < npts, nmo <= 0)");
    if (((uintptr_t)d_qt & 15) != 0) return set_error(OKG_ERR_ARG, "okg_ci_flux_matrix: d_qt not 16-byte aligned");
    if (npts == 0) return OKG_OK;
    const unsigned nblk = (unsigned)((npts + 127) / 128);
    ci_quad_kernel<true><<<nblk, 128, 0, (cudaStream_t)stream>>>(npts, d_mo, d_drv, ld, nmo, d_qt, scale, d_j);
    return cuda_status(cudaGetLastError(), "okg_ci_flux_matrix launch");
}
