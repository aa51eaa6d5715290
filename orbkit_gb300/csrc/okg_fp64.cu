// FP64 fused AO -> MO -> density kernels (okg_eval_mo, okg_rho); the AO
// kernels of okg_eval_ao are in okg_ao.cu.
//
// Reference algorithm: orbkit/c_grid-based.c:9-79 (c_lcreator: per point, per
// primitive exp, per Cartesian component the contraction times the polynomial or
// the derivative factor of orbkit/c_support.c:28-175), orbkit/cy_core.pyx:82-101
// (mocreator) and orbkit/core.py:266-304 (density and its derivatives).
//
// Layout in HBM: AO / MO outputs are row-major (slot, row, point) with points
// contiguous -- the reference's ao_list[k, i] -- so every warp writes 32
// consecutive doubles.  Regular grids are never flattened in memory: a point's
// coordinates come from its flattened index (x slowest, z fastest).
#include <stdio.h>

#include "okg_internal.cuh"

namespace okg {

// ------------------------------------------------------------- fused kernels
// CTA = FP points x FG MO groups (64 x 4 = 256 threads; 8 x 16 for small point
// sets).  For each chunk of shells, every
// group evaluates a share of the chunk's shells for its point into shared memory
// (AO_s[channel][row][point], NCH channels = the first NCH of value, d/dx, d/dy,
// d/dz, xx, yy, zz, xy, xz, yz); the chunk's MO coefficients are staged in C_s;
// then each thread accumulates MB MOs x NCH channels for its point in registers.
// The AO and MO values never leave the SM.  MO counts above G*MB are handled by
// passes over MO blocks (AO values are re-evaluated per pass).
constexpr int FP = 64;   // points per CTA
constexpr int FG = 4;    // MO groups
constexpr int FT = FP * FG;

struct FusedArgs {
    int nmo;
    const double* C;    // nmo x ncart
    const double* occ;  // nmo
    DrvList drv;
    int mixed_ref;
    double* out;        // MO mode: ndrv x nmo x ld ; rho mode: rho (ld)
    double* dout;       // rho mode: ndrv x ld
    double* mo_norm;    // rho mode: nmo or null
    long long ld;
};

template <int NCH>
__device__ __forceinline__ double pick(const double (&v)[NCH], int c)
{
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < NCH; ++i) r = (i == c) ? v[i] : r;
    return r;
}

__host__ __device__ inline void second_pair(int code, int& a, int& b)
{
    // first-derivative channels whose product enters the two-letter term
    switch (code) {
    case 4: a = 1; b = 1; break;
    case 5: a = 2; b = 2; break;
    case 6: a = 3; b = 3; break;
    case 7: a = 1; b = 2; break;
    case 8: a = 1; b = 3; break;
    case 9: a = 2; b = 3; break;
    default: a = b = 0; break;
    }
}

template <int NCH, int MB, bool MO_OUT, int FP = okg::FP, int FG = okg::FG>
__global__ void __launch_bounds__(FP * FG) fused64_kernel(BasisDev B, Grid g, FusedArgs A)
{
    constexpr int FT = FP * FG;
    extern __shared__ double smem[];
    double* AO_s = smem;                          // NCH x KC x FP
    double* C_s = smem + NCH * OKG_KC * FP;       // FG*MB x KC
    const int tid = threadIdx.x;
    const int pl = tid % FP;
    const int grp = tid / FP;
    const long long p = (long long)blockIdx.x * FP + pl;
    const bool valid = p < g.npts;
    double x, y, z;
    grid_point(g, valid ? p : g.npts - 1, x, y, z);
    constexpr unsigned chmask = (1u << NCH) - 1u;
    constexpr int MOPASS = FG * MB;

    double rho_part = 0.0;
    double drho_part[10];
#pragma unroll
    for (int d = 0; d < 10; ++d) drho_part[d] = 0.0;

    for (int mo0 = 0; mo0 < A.nmo; mo0 += MOPASS) {
        double acc[MB][NCH];
#pragma unroll
        for (int m = 0; m < MB; ++m)
#pragma unroll
            for (int c = 0; c < NCH; ++c) acc[m][c] = 0.0;

        for (int ci = 0; ci < B.nchunk; ++ci) {
            const int4 ck = B.chunks[ci];
            const int kc = ck.w - ck.z;
            __syncthreads();  // previous chunk fully consumed
            for (int i = tid; i < MOPASS * OKG_KC; i += FT) {
                const int m = i / OKG_KC, kk = i % OKG_KC;
                const int mo = mo0 + m;
                C_s[i] = (mo < A.nmo && kk < kc) ? A.C[(long long)mo * B.ncart + ck.z + kk] : 0.0;
            }
            int last_atom = -1;
            double X = 0, Y = 0, Z = 0, rr = 0;
            for (int s = ck.x + grp; s < ck.y; s += FG) {
                const Shell sh = B.shells[s];
                if (sh.atom != last_atom) {
                    X = x - B.atoms[4 * sh.atom];
                    Y = y - B.atoms[4 * sh.atom + 1];
                    Z = z - B.atoms[4 * sh.atom + 2];
                    rr = X * X + Y * Y + Z * Z;
                    last_atom = sh.atom;
                }
                const Radial<double> r = radial64(B.prim, sh.prim0, sh.nprim, rr, NCH > 1, NCH > 4);
                const int rowbase = sh.cart0 - ck.z;
                shell_eval_L(sh.L, X, Y, Z, r, chmask, A.mixed_ref != 0, [&](int ch, int j, double v) {
                    const int row = B.comp_row[sh.comp0 + j];
                    if (row < 0) return;
                    AO_s[(ch * OKG_KC + rowbase + row) * FP + pl] = v * B.comp_g[sh.comp0 + j];
                });
            }
            __syncthreads();
            const double* Cg = C_s + grp * MB * OKG_KC;
            for (int kk = 0; kk < kc; ++kk) {
                double a[NCH];
#pragma unroll
                for (int c = 0; c < NCH; ++c) a[c] = AO_s[(c * OKG_KC + kk) * FP + pl];
#pragma unroll
                for (int m = 0; m < MB; ++m) {
                    const double cm = Cg[m * OKG_KC + kk];
#pragma unroll
                    for (int c = 0; c < NCH; ++c) acc[m][c] = fma(cm, a[c], acc[m][c]);
                }
            }
        }

        // epilogue of this MO pass
#pragma unroll
        for (int m = 0; m < MB; ++m) {
            const int mo = mo0 + grp * MB + m;
            if (mo >= A.nmo) break;
            if (MO_OUT) {
                if (valid)
                    for (int d = 0; d < A.drv.n; ++d)
                        A.out[((long long)d * A.nmo + mo) * A.ld + p] = pick<NCH>(acc[m], A.drv.code[d]);
            } else {
                const double o = A.occ[mo];
                const double v0 = acc[m][0];
                rho_part += o * (v0 * v0);
                const double o2 = o * 2;
#pragma unroll
                for (int d = 0; d < 10; ++d) {
                    if (d >= A.drv.n) break;
                    const int code = A.drv.code[d];
                    double t = (o2 * pick<NCH>(acc[m], code)) * v0;
                    if (code >= 4) {
                        int ca, cb;
                        second_pair(code, ca, cb);
                        t += o2 * (pick<NCH>(acc[m], ca) * pick<NCH>(acc[m], cb));
                    }
                    drho_part[d] += t;
                }
                if (A.mo_norm) {
                    double q = valid ? v0 * v0 : 0.0;
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
                    if ((tid & 31) == 0) atomicAdd(A.mo_norm + mo, q);
                }
            }
        }
    }

    if (!MO_OUT) {
        // reduce the FG group partials per point, in fixed order
        __syncthreads();
        double* red = smem;  // FG x (1 + 10) x FP
        red[(grp * 11 + 0) * FP + pl] = rho_part;
#pragma unroll
        for (int d = 0; d < 10; ++d)
            if (d < A.drv.n) red[(grp * 11 + 1 + d) * FP + pl] = drho_part[d];
        __syncthreads();
        if (grp == 0 && valid) {
            double r = 0.0;
            for (int q = 0; q < FG; ++q) r += red[(q * 11) * FP + pl];
            A.out[p] = r;
            for (int d = 0; d < A.drv.n; ++d) {
                double t = 0.0;
                for (int q = 0; q < FG; ++q) t += red[(q * 11 + 1 + d) * FP + pl];
                A.dout[(long long)d * A.ld + p] = t;
            }
        }
    }
}

template <int NCH, int MB, bool MO_OUT, int FPx = FP, int FGx = FG>
static int launch_fused(const okg_basis* b, const Grid& g, const FusedArgs& A, cudaStream_t st)
{
    const size_t smem_main = sizeof(double) * ((size_t)NCH * OKG_KC * FPx + (size_t)FGx * MB * OKG_KC);
    const size_t smem_red = sizeof(double) * FGx * 11 * FPx;
    const size_t smem = smem_main > smem_red ? smem_main : smem_red;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(fused64_kernel<NCH, MB, MO_OUT, FPx, FGx>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "fused64: smem attribute");
        configured = true;
    }
    const long long nblk = (g.npts + FPx - 1) / FPx;
    fused64_kernel<NCH, MB, MO_OUT, FPx, FGx><<<(unsigned)nblk, FPx * FGx, smem, st>>>(b->dev, g, A);
    return cuda_status(cudaGetLastError(), "fused64 launch");
}

// Small point sets -- fewer than one wave of the 64-point CTAs, e.g. the FP64
// recomputation of the points near nuclei on the mixed path -- use CTAs of 8
// points x 16 MO groups: the same kernel and per-point arithmetic, 8x as many
// CTAs, every lane busy in the AO and in the MO part (measured faster than 2 x 64
// on 678 points: more CTAs restage the coefficients more often).
constexpr long long FEW_MAX_POINTS = 152 * FP;

static int dispatch_few(const okg_basis* b, const Grid& g, const FusedArgs& A, unsigned need, cudaStream_t st)
{
    if ((need & ~1u) == 0) return launch_fused<1, 8, false, 8, 16>(b, g, A, st);
    if ((need & ~0xFu) == 0) return launch_fused<4, 4, false, 8, 16>(b, g, A, st);
    if ((need & ~0x7Fu) == 0) return launch_fused<7, 3, false, 8, 16>(b, g, A, st);
    return launch_fused<10, 2, false, 8, 16>(b, g, A, st);
}

template <bool MO_OUT>
static int dispatch_fused(const okg_basis* b, const Grid& g, const FusedArgs& A, unsigned need, cudaStream_t st)
{
    if ((need & ~1u) == 0) return launch_fused<1, 32, MO_OUT>(b, g, A, st);
    if ((need & ~0xFu) == 0) return launch_fused<4, 10, MO_OUT>(b, g, A, st);
    if ((need & ~0x7Fu) == 0) return launch_fused<7, 6, MO_OUT>(b, g, A, st);
    return launch_fused<10, 4, MO_OUT>(b, g, A, st);
}

}  // namespace okg

using namespace okg;

extern "C" int okg_eval_mo(const okg_basis* b, const okg_grid* grid, int nmo, const double* d_coeff, int ndrv,
                           const int* h_drv, int exact_mixed, double* d_out, int64_t ld, okg_stream stream)
{
    if (!b || !d_out || !d_coeff || nmo <= 0) return set_error(OKG_ERR_ARG, "okg_eval_mo: NULL argument or nmo <= 0");
    Grid g;
    int st = make_grid(grid, g);
    if (st) return st;
    FusedArgs A{};
    unsigned mask;
    if ((st = make_drv(ndrv, h_drv, A.drv, mask))) return st;
    if (ndrv == 0 || g.npts == 0) return OKG_OK;
    if (ld < g.npts) return set_error(OKG_ERR_ARG, "okg_eval_mo: ld < npts");
    A.nmo = nmo;
    A.C = d_coeff;
    A.mixed_ref = !exact_mixed;
    A.out = d_out;
    A.ld = ld;
    return dispatch_fused<true>(b, g, A, mask | 1u, (cudaStream_t)stream);
}

extern "C" int okg_rho(const okg_basis* b, const okg_grid* grid, int nmo, const double* d_coeff, const double* d_occ,
                       int ndrv, const int* h_drv, int exact_mixed, double* d_rho, double* d_drho, int64_t ld,
                       double* d_mo_norm, okg_stream stream)
{
    if (!b || !d_rho || !d_coeff || !d_occ || nmo <= 0)
        return set_error(OKG_ERR_ARG, "okg_rho: NULL argument or nmo <= 0");
    Grid g;
    int st = make_grid(grid, g);
    if (st) return st;
    FusedArgs A{};
    unsigned mask;
    if ((st = make_drv(ndrv, h_drv, A.drv, mask))) return st;
    if (ndrv > 0 && !d_drho) return set_error(OKG_ERR_ARG, "okg_rho: d_drho is NULL");
    if (g.npts == 0) return OKG_OK;
    if (ld < g.npts) return set_error(OKG_ERR_ARG, "okg_rho: ld < npts");
    unsigned need = 1u;
    for (int i = 0; i < ndrv; ++i) {
        need |= 1u << A.drv.code[i];
        if (A.drv.code[i] >= 4) {
            int a, c;
            second_pair(A.drv.code[i], a, c);
            need |= (1u << a) | (1u << c);
        }
    }
    A.nmo = nmo;
    A.C = d_coeff;
    A.occ = d_occ;
    A.mixed_ref = !exact_mixed;
    A.out = d_rho;
    A.dout = d_drho;
    A.mo_norm = d_mo_norm;
    A.ld = ld;
    // (the MO-norm sums reduce over warps of one MO group: 64-point CTAs only)
    if (g.npts <= FEW_MAX_POINTS && !A.mo_norm) return dispatch_few(b, g, A, need, (cudaStream_t)stream);
    return dispatch_fused<false>(b, g, A, need, (cudaStream_t)stream);
}
