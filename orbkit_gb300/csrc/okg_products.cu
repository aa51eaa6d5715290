// Grid-array operations on given AO / MO values (FP64):
//
//   okg_mo_from_ao    MO = C . AO                 orbkit/cy_core.pyx:82-101 (mocreator),
//                                                 behind core.mo_creator (orbkit/core.py:107-132)
//   okg_cart2sph      spherical rows from the      orbkit/core.py:135-176 (cartesian2spherical)
//                     Cartesian rows (CSR)
//   okg_mo_products   MO_a(r) * dMO_b(r)          orbkit/core.py:935-937 (calc_mo_matrix)
//   okg_mo_pair_flux  -1/2 (MO_i dMO_j - MO_j dMO_i)  orbkit/extras.py:484-487 (calc_jmo)
//
// Layout: every array is row-major (row, point) with points contiguous and a
// leading dimension per array (orbkit's ao_list[k, i] / mo_list[m, i]), so every
// warp reads and writes 32 consecutive doubles of a row.
//
// okg_mo_from_ao is bound by the FP64 pipe (GB300: 2 DFMA per clock per SM): a CTA
// covers 64 points x up to 64 MOs, the coefficients of a 32-AO chunk are staged in
// shared memory and read as warp-wide broadcasts, each AO value is loaded once per
// (point, MO group) and used for MB FMAs from registers.  The three others are
// HBM-bound streams: one multiply (products) or two multiplies, a subtraction and
// a scaling (pair flux) per output element, rounded exactly as numpy rounds them
// (no FMA contraction), so their results equal orbkit's bit for bit for the same
// MO grids; the CSR transform adds its terms in orbkit's order with orbkit's
// rounding, likewise bit for bit.
#include "okg_internal.cuh"

namespace okg {
namespace prod {

constexpr int GP = 64;   // points per CTA of the contraction
constexpr int GG = 4;    // MO groups per CTA
constexpr int GK = 32;   // AOs per staged coefficient chunk

// out[m, i] = sum_k C[m, k] A[k, i] for the MOs [mo0, mo0 + GG*MB) of blockIdx.y.
template <int MB>
__global__ void __launch_bounds__(GP * GG) mo_from_ao_kernel(int nmo, int nao, const double* __restrict__ C,
                                                              const double* __restrict__ A, long long lda,
                                                              long long npts, double* __restrict__ out, long long ldo)
{
    __shared__ double C_s[GK][GG * MB];  // chunk of coefficients, k-major: a warp reads one address
    const int tid = threadIdx.x;
    const int pl = tid % GP, grp = tid / GP;
    const long long p = (long long)blockIdx.x * GP + pl;
    const bool valid = p < npts;
    const int mo0 = blockIdx.y * GG * MB;
    double acc[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) acc[m] = 0.0;
    const double* a_col = A + (valid ? p : 0);
    for (int k0 = 0; k0 < nao; k0 += GK) {
        const int kc = nao - k0 < GK ? nao - k0 : GK;
        __syncthreads();
        for (int i = tid; i < GK * GG * MB; i += GP * GG) {
            const int kk = i / (GG * MB), m = i % (GG * MB);
            const int mo = mo0 + m;
            C_s[kk][m] = (kk < kc && mo < nmo) ? C[(long long)mo * nao + k0 + kk] : 0.0;
        }
        __syncthreads();
        const double* ap = a_col + (long long)k0 * lda;
        int kk = 0;
        // four AO values in flight per thread
        for (; kk + 4 <= kc; kk += 4) {
            double a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = valid ? __ldg(ap + (long long)(kk + u) * lda) : 0.0;
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int m = 0; m < MB; ++m) acc[m] = fma(C_s[kk + u][grp * MB + m], a[u], acc[m]);
        }
        for (; kk < kc; ++kk) {
            const double a = valid ? __ldg(ap + (long long)kk * lda) : 0.0;
#pragma unroll
            for (int m = 0; m < MB; ++m) acc[m] = fma(C_s[kk][grp * MB + m], a, acc[m]);
        }
    }
    if (!valid) return;
#pragma unroll
    for (int m = 0; m < MB; ++m) {
        const int mo = mo0 + grp * MB + m;
        if (mo < nmo) out[(long long)mo * ldo + p] = acc[m];
    }
}

template <int MB>
static int launch_mo_from_ao(int nmo, int nao, const double* C, const double* A, long long lda, long long npts,
                             double* out, long long ldo, cudaStream_t st)
{
    const long long bx = (npts + GP - 1) / GP;
    const int by = (nmo + GG * MB - 1) / (GG * MB);
    if (bx > 0x7FFFFFFFll || by > 65535) return set_error(OKG_ERR_UNSUPPORTED, "okg_mo_from_ao: grid too large");
    mo_from_ao_kernel<MB><<<dim3((unsigned)bx, (unsigned)by), GP * GG, 0, st>>>(nmo, nao, C, A, lda, npts, out, ldo);
    return cuda_status(cudaGetLastError(), "okg_mo_from_ao launch");
}

// Rows handed out over gridDim.y (with a stride, so any row count works), points
// over gridDim.x with a stride.
constexpr int SP = 256;

__global__ void __launch_bounds__(SP) cart2sph_kernel(int nsph, int ncart, const int* __restrict__ ptr,
                                                      const int* __restrict__ cart, const double* __restrict__ coef,
                                                      const double* __restrict__ in, long long ldi, long long npts,
                                                      double* __restrict__ out, long long ldo)
{
    for (int r = blockIdx.y; r < nsph; r += gridDim.y) {
        const int t0 = __ldg(ptr + r), t1 = __ldg(ptr + r + 1);
        for (long long p = (long long)blockIdx.x * SP + threadIdx.x; p < npts; p += (long long)gridDim.x * SP) {
            double acc = 0.0;
            for (int t = t0; t < t1; ++t) {
                const int c = __ldg(cart + t);
                // a component row outside the input: NaN, no access
                const double v = (c >= 0 && c < ncart) ? __ldg(in + (long long)c * ldi + p)
                                                      : __longlong_as_double(0x7FF8000000000000ll);
                acc = __dadd_rn(acc, __dmul_rn(__ldg(coef + t), v));
            }
            out[(long long)r * ldo + p] = acc;
        }
    }
}

__global__ void __launch_bounds__(SP) mo_products_kernel(int ndrv, int na, int nb, const double* __restrict__ bra,
                                                         long long ldb, const double* __restrict__ ket, long long ldk,
                                                         long long npts, double* __restrict__ out, long long ldo)
{
    const long long rows = (long long)ndrv * na * nb;
    for (long long r = blockIdx.y; r < rows; r += gridDim.y) {
        const int m = (int)(r % nb);
        const int n = (int)((r / nb) % na);
        const int d = (int)(r / ((long long)nb * na));
        const double* b = bra + (long long)n * ldb;
        const double* k = ket + ((long long)d * nb + m) * ldk;
        double* o = out + r * ldo;
        for (long long p = (long long)blockIdx.x * SP + threadIdx.x; p < npts; p += (long long)gridDim.x * SP)
            o[p] = __dmul_rn(__ldg(b + p), __ldg(k + p));
    }
}

__global__ void __launch_bounds__(SP) mo_pair_flux_kernel(int ndrv, int nmo, int npair, const int* __restrict__ pairs,
                                                          const double* __restrict__ bra, long long ldb,
                                                          const double* __restrict__ ket, long long ldk,
                                                          long long npts, double* __restrict__ out, long long ldo)
{
    const long long rows = (long long)ndrv * npair;
    for (long long r = blockIdx.y; r < rows; r += gridDim.y) {
        const int q = (int)(r % npair);
        const int d = (int)(r / npair);
        const int i = __ldg(pairs + 2 * q), j = __ldg(pairs + 2 * q + 1);
        double* o = out + r * ldo;
        if (i < 0 || i >= nmo || j < 0 || j >= nmo) {  // an index outside the MO grids: NaN, no access
            for (long long p = (long long)blockIdx.x * SP + threadIdx.x; p < npts; p += (long long)gridDim.x * SP)
                o[p] = __longlong_as_double(0x7FF8000000000000ll);
            continue;
        }
        const double* bi = bra + (long long)i * ldb;
        const double* bj = bra + (long long)j * ldb;
        const double* ki = ket + ((long long)d * nmo + i) * ldk;
        const double* kj = ket + ((long long)d * nmo + j) * ldk;
        for (long long p = (long long)blockIdx.x * SP + threadIdx.x; p < npts; p += (long long)gridDim.x * SP) {
            const double ij = __dmul_rn(__ldg(bi + p), __ldg(kj + p));
            const double ji = __dmul_rn(__ldg(bj + p), __ldg(ki + p));
            o[p] = __dmul_rn(-0.5, __dsub_rn(ij, ji));
        }
    }
}

// Launch shape of the streaming kernels: enough point blocks for a few waves of
// 152 SMs, rows over y (at most 65535, strided beyond).
static dim3 stream_grid(long long npts, long long rows)
{
    long long bx = (npts + SP - 1) / SP;
    long long by = rows < 65535 ? rows : 65535;
    // keep total CTAs bounded for very long rows: strided loops cover the rest
    const long long cap = 152ll * 8 * 64;
    if (bx * by > cap) bx = cap / by > 0 ? cap / by : 1;
    return dim3((unsigned)(bx > 0 ? bx : 1), (unsigned)(by > 0 ? by : 1));
}

}  // namespace prod
}  // namespace okg

using namespace okg;

extern "C" int okg_mo_from_ao(int nmo, int nao, const double* d_coeff, const double* d_ao, int64_t ld_ao,
                              int64_t npts, double* d_out, int64_t ld_out, okg_stream stream)
{
    if (nmo <= 0 || nao <= 0 || !d_coeff || !d_ao || !d_out || npts < 0)
        return set_error(OKG_ERR_ARG, "okg_mo_from_ao: NULL pointer, nmo <= 0, nao <= 0 or npts < 0");
    if (ld_ao < npts || ld_out < npts) return set_error(OKG_ERR_ARG, "okg_mo_from_ao: leading dimension < npts");
    if (npts == 0) return OKG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (nmo <= 4) return prod::launch_mo_from_ao<1>(nmo, nao, d_coeff, d_ao, ld_ao, npts, d_out, ld_out, st);
    if (nmo <= 8) return prod::launch_mo_from_ao<2>(nmo, nao, d_coeff, d_ao, ld_ao, npts, d_out, ld_out, st);
    if (nmo <= 16) return prod::launch_mo_from_ao<4>(nmo, nao, d_coeff, d_ao, ld_ao, npts, d_out, ld_out, st);
    if (nmo <= 32) return prod::launch_mo_from_ao<8>(nmo, nao, d_coeff, d_ao, ld_ao, npts, d_out, ld_out, st);
    return prod::launch_mo_from_ao<16>(nmo, nao, d_coeff, d_ao, ld_ao, npts, d_out, ld_out, st);
}

extern "C" int okg_cart2sph(int nsph, int ncart, const int* d_ptr, const int* d_cart, const double* d_coef,
                            const double* d_in, int64_t ld_in, int64_t npts, double* d_out, int64_t ld_out,
                            okg_stream stream)
{
    if (nsph <= 0 || ncart <= 0 || !d_ptr || !d_cart || !d_coef || !d_in || !d_out || npts < 0)
        return set_error(OKG_ERR_ARG, "okg_cart2sph: NULL pointer, nsph <= 0, ncart <= 0 or npts < 0");
    if (ld_in < npts || ld_out < npts) return set_error(OKG_ERR_ARG, "okg_cart2sph: leading dimension < npts");
    if (npts == 0) return OKG_OK;
    prod::cart2sph_kernel<<<prod::stream_grid(npts, nsph), prod::SP, 0, (cudaStream_t)stream>>>(
        nsph, ncart, d_ptr, d_cart, d_coef, d_in, ld_in, npts, d_out, ld_out);
    return cuda_status(cudaGetLastError(), "okg_cart2sph launch");
}

extern "C" int okg_mo_products(int ndrv, int na, int nb, const double* d_bra, int64_t ld_bra, const double* d_ket,
                               int64_t ld_ket, int64_t npts, double* d_out, int64_t ld_out, okg_stream stream)
{
    if (ndrv <= 0 || na <= 0 || nb <= 0 || !d_bra || !d_ket || !d_out || npts < 0)
        return set_error(OKG_ERR_ARG, "okg_mo_products: NULL pointer, a count <= 0 or npts < 0");
    if (ld_bra < npts || ld_ket < npts || ld_out < npts)
        return set_error(OKG_ERR_ARG, "okg_mo_products: leading dimension < npts");
    if (npts == 0) return OKG_OK;
    prod::mo_products_kernel<<<prod::stream_grid(npts, (long long)ndrv * na * nb), prod::SP, 0, (cudaStream_t)stream>>>(
        ndrv, na, nb, d_bra, ld_bra, d_ket, ld_ket, npts, d_out, ld_out);
    return cuda_status(cudaGetLastError(), "okg_mo_products launch");
}

extern "C" int okg_mo_pair_flux(int ndrv, int nmo, int npair, const int* d_pairs, const double* d_bra, int64_t ld_bra,
                                const double* d_ket, int64_t ld_ket, int64_t npts, double* d_out, int64_t ld_out,
                                okg_stream stream)
{
    if (ndrv <= 0 || nmo <= 0 || npair <= 0 || !d_pairs || !d_bra || !d_ket || !d_out || npts < 0)
        return set_error(OKG_ERR_ARG, "okg_mo_pair_flux: NULL pointer, a count <= 0 or npts < 0");
    if (ld_bra < npts || ld_ket < npts || ld_out < npts)
        return set_error(OKG_ERR_ARG, "okg_mo_pair_flux: leading dimension < npts");
    if (npts == 0) return OKG_OK;
    prod::mo_pair_flux_kernel<<<prod::stream_grid(npts, (long long)ndrv * npair), prod::SP, 0,
                                (cudaStream_t)stream>>>(ndrv, nmo, npair, d_pairs, d_bra, ld_bra, d_ket, ld_ket, npts,
                                                        d_out, ld_out);
    return cuda_status(cudaGetLastError(), "okg_mo_pair_flux launch");
}
