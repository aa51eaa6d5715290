// AO values and AO derivatives on a grid, FP64 (okg_eval_ao).
//
// Reference: orbkit/c_grid-based.c:9-79 (c_lcreator: per point and primitive
// exp(-alpha r^2), per Cartesian component the contraction times the polynomial or
// the derivative factor of orbkit/c_support.c:28-175), followed by the 'N' factor and
// cartesian2spherical (orbkit/core.py:89-102).  Per (shell, point) the primitive
// exponentials are reduced to the radial sums R0, R1, R2 once; every requested
// derivative code and every component is then a short polynomial of them
// (okg_internal.cuh), so exp, the polynomial and the contraction run once per
// (shell, point) whatever the number of drv codes.
//
// Regular grids (ao_tile_kernel): a CTA covers 8 grid lines (fixed x and y, one
// per warp) x 32 consecutive z (one per lane): every warp writes 32 consecutive
// doubles of each output row.  The Gaussian separates along the axes,
// exp(-a (X^2 + Y^2 + Z^2)) = exp(-a (X^2 + Y^2)) exp(-a Z^2), so for a window of
// up to 64 primitives the CTA tabulates w exp(-a (X^2 + Y^2)) for its 8 lines and
// exp(-a Z^2) for its 32 z in shared memory (40 exponentials per primitive for 256
// points) and a point's primitive term is one product of two table entries.  The
// factorised exponential differs from exp of the summed argument by a few units
// in the last place, far inside the FP64 parity bar.
//
// Vector grids (ao_point_kernel): one point per thread, the primitives of the
// current window staged in shared memory, exp per (primitive, point).
//
// Both stage the shell records (windows of 64 shells) and the primitives
// (exponent, weight) in shared memory; spherical outputs take the shell's
// Cartesian values from a per-thread shared-memory column (no local arrays).
// Shells with more primitives than one window evaluate their exponentials per
// point.
#include "okg_internal.cuh"

namespace okg {
namespace ao {

constexpr int NT = 256;           // threads per CTA (8 warps)
constexpr int LINES = 8;          // regular grids: grid lines per CTA, one per warp
constexpr int ZB = 32;            // regular grids: consecutive z per CTA, one per lane
constexpr int PW = 64;            // primitives per staged window
constexpr int SW = 64;            // shell records per staged window
constexpr int TW = LINES + ZB;    // table entries per primitive

// Shared-memory carve-up (bytes), 16-byte aligned pieces.
constexpr size_t OFF_TXY = 0;                                    // PW x LINES doubles
constexpr size_t OFF_TZ = OFF_TXY + sizeof(double) * PW * LINES;  // PW x ZB doubles
constexpr size_t OFF_PA = OFF_TZ + sizeof(double) * PW * ZB;      // PW x 2 doubles: alpha, w
constexpr size_t OFF_SH = OFF_PA + sizeof(double) * PW * 2;       // SW shells
constexpr size_t OFF_CODE = OFF_SH + sizeof(Shell) * SW;          // 16 ints: drv codes
constexpr size_t OFF_CV = OFF_CODE + 64;                          // spherical: 15 x NT doubles
constexpr size_t SMEM_CART = OFF_CV;
constexpr size_t SMEM_SPH = OFF_CV + sizeof(double) * OKG_MAX_NCART * NT;
static_assert(OFF_CV % 16 == 0 && OFF_SH % 16 == 0, "shared-memory pieces must stay 16-byte aligned");

struct Tables {
    double (*txy)[LINES];
    double (*tz)[ZB];
    double* pa;      // alpha, w per window primitive
    Shell* sh;       // window of shell records
    int* code;       // drv codes (-1 beyond ndrv)
    double* cv;      // spherical: canonical values, [component][thread]
};

__device__ __forceinline__ Tables carve(unsigned char* smem)
{
    Tables t;
    t.txy = (double(*)[LINES])(smem + OFF_TXY);
    t.tz = (double(*)[ZB])(smem + OFF_TZ);
    t.pa = (double*)(smem + OFF_PA);
    t.sh = (Shell*)(smem + OFF_SH);
    t.code = (int*)(smem + OFF_CODE);
    t.cv = (double*)(smem + OFF_CV);
    return t;
}

// One shell's outputs at this thread's point: the channels of chmask from the
// radial sums, into every drv slot that asks for them (Cartesian rows scaled by the
// angular norm x 'N'; spherical rows through the shell's transform).
template <bool SPH>
__device__ __forceinline__ void write_shell(const BasisDev& B, const Shell& sh, const Tables& T, double X, double Y,
                                            double Z, const Radial<double>& r, unsigned chmask, int ndrv,
                                            bool mixed_ref, bool valid, double* __restrict__ out, long long ld,
                                            long long p, int nao)
{
    if (!SPH) {
        shell_eval_L(sh.L, X, Y, Z, r, chmask, mixed_ref, [&](int ch, int j, double v) {
            const int row = __ldg(B.comp_row + sh.comp0 + j);
            if (row < 0 || !valid) return;
            const double gv = v * __ldg(B.comp_g + sh.comp0 + j);
            for (int d = 0; d < ndrv; ++d)
                if (T.code[d] == ch) out[((long long)d * nao + sh.out0 + row) * ld + p] = gv;
        });
    } else {
        double* cv = T.cv + threadIdx.x;
        for (int ch = 0; ch < 10; ++ch) {
            if (!(chmask & (1u << ch))) continue;
            shell_eval_L(sh.L, X, Y, Z, r, 1u << ch, mixed_ref,
                         [&](int, int j, double v) { cv[j * NT] = v * __ldg(B.comp_g + sh.comp0 + j); });
            if (!valid) continue;
            for (int o = 0; o < sh.nout; ++o) {
                const int row = sh.sph0 + o;
                double acc = 0.0;
                const int t1 = __ldg(B.sph_ptr + row + 1);
                for (int t = __ldg(B.sph_ptr + row); t < t1; ++t)
                    acc += __ldg(B.sph_coef + t) * cv[__ldg(B.sph_cidx + t) * NT];
                for (int d = 0; d < ndrv; ++d)
                    if (T.code[d] == ch) out[((long long)d * nao + row) * ld + p] = acc;
            }
        }
    }
}

// Shell window: records [s0, s0 + SW) into shared memory (CTA-uniform call).
__device__ __forceinline__ void stage_shells(const BasisDev& B, const Tables& T, int s0)
{
    __syncthreads();
    constexpr int U = (int)(sizeof(Shell) / 4);
    const int n = (B.nshell - s0 < SW ? B.nshell - s0 : SW) * U;
    const int* src = (const int*)(B.shells + s0);
    int* dst = (int*)T.sh;
    for (int i = threadIdx.x; i < n; i += NT) dst[i] = __ldg(src + i);
    __syncthreads();
}

// Regular grid: CTA = LINES lines x ZB z of the lines [line0, ...) of the call.
template <bool SPH, unsigned UB>
__global__ void __launch_bounds__(NT, UB == 1u ? 2 : 1) ao_tile_kernel(BasisDev B, Grid g, DrvList drv, unsigned chmask_in, int mixed_ref,
                                                     double* __restrict__ out, long long ld, int nao, long long line0,
                                                     int nzb)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const Tables T = carve(smem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long lg = blockIdx.x / nzb;
    const int kb = (int)(blockIdx.x - lg * nzb);
    const long long nlines = (long long)g.nx * g.ny;
    const long long lbase = line0 + lg * LINES;  // first line of the CTA
    const long long line = lbase + warp;
    const int k = kb * ZB + lane;
    const long long flat = line * g.nz + k;
    const bool valid = line < nlines && k < g.nz && flat >= g.offset && flat < g.offset + g.npts;
    const long long p = valid ? flat - g.offset : 0;
    double x = 0.0, y = 0.0, z = 0.0;
    if (line < nlines) {
        const int i = (int)(line / g.ny);
        x = __ldg(g.x + i);
        y = __ldg(g.y + (int)(line - (long long)i * g.ny));
    }
    if (k < g.nz) z = __ldg(g.z + k);
    if (tid < 16) T.code[tid] = tid < drv.n ? drv.code[tid] : -1;
    // UB: the channels this instantiation can produce (value; value and first
    // derivatives; all), so that the others are compiled out
    const unsigned chmask = UB == 1u ? 1u : (chmask_in & UB);
    const bool n1 = need_r1(chmask), n2 = need_r2(chmask);
    int w0 = 0, wn = 0, s0 = -SW;
    int last_atom = -1;
    double X = 0.0, Y = 0.0, Z = 0.0, rr = 0.0;
    for (int s = 0; s < B.nshell; ++s) {
        if (s >= s0 + SW) {
            s0 = s;
            stage_shells(B, T, s0);
        }
        const Shell sh = T.sh[s - s0];
        const bool tab = sh.nprim <= PW;
        if (tab && (sh.prim0 < w0 || sh.prim0 + sh.nprim > w0 + wn)) {
            // refill the primitive window from this shell on: per primitive, w exp(-a (X^2 + Y^2))
            // for the CTA's lines and exp(-a Z^2) for its z
            __syncthreads();
            w0 = sh.prim0;
            wn = B.nprim - w0 < PW ? B.nprim - w0 : PW;
            for (int e = tid; e < wn * TW; e += NT) {
                const int q = e / TW, t = e - q * TW;
                const int P = w0 + q;
                const double a = __ldg(B.prim + 2 * P), w = __ldg(B.prim + 2 * P + 1);
                const int at = __ldg(B.prim_atom + P);
                double v = 0.0;
                if (t < LINES) {
                    const long long ln = lbase + t;
                    if (ln < nlines) {
                        const int i = (int)(ln / g.ny);
                        const double Xa = __ldg(g.x + i) - __ldg(B.atoms + 4 * at);
                        const double Ya = __ldg(g.y + (int)(ln - (long long)i * g.ny)) - __ldg(B.atoms + 4 * at + 1);
                        v = w * exp(-a * (Xa * Xa + Ya * Ya));
                    }
                    T.txy[q][t] = v;
                } else {
                    const int kk = kb * ZB + (t - LINES);
                    if (kk < g.nz) {
                        const double Za = __ldg(g.z + kk) - __ldg(B.atoms + 4 * at + 2);
                        v = exp(-a * (Za * Za));
                    }
                    T.tz[q][t - LINES] = v;
                }
                if (t == 0) {
                    T.pa[2 * q] = a;
                    T.pa[2 * q + 1] = w;
                }
            }
            __syncthreads();
        }
        if (sh.atom != last_atom) {
            last_atom = sh.atom;
            X = x - __ldg(B.atoms + 4 * sh.atom);
            Y = y - __ldg(B.atoms + 4 * sh.atom + 1);
            Z = z - __ldg(B.atoms + 4 * sh.atom + 2);
            rr = X * X + Y * Y + Z * Z;
        }
        Radial<double> r{0.0, 0.0, 0.0};
        if (tab) {
            const int q0 = sh.prim0 - w0;
            for (int q = q0; q < q0 + sh.nprim; ++q) {
                const double e = T.txy[q][warp] * T.tz[q][lane];
                r.R0 += e;
                if (n1) r.R1 += T.pa[2 * q] * e;
                if (n2) r.R2 += T.pa[2 * q] * T.pa[2 * q] * e;
            }
        } else {
            r = radial64(B.prim, sh.prim0, sh.nprim, rr, n1, n2);
        }
        write_shell<SPH>(B, sh, T, X, Y, Z, r, chmask, drv.n, mixed_ref != 0, valid, out, ld, p, nao);
    }
}

// Vector grid: one point per thread, primitive windows staged in shared memory.
template <bool SPH, unsigned UB>
__global__ void __launch_bounds__(NT, UB == 1u ? 2 : 1) ao_point_kernel(BasisDev B, Grid g, DrvList drv, unsigned chmask_in, int mixed_ref,
                                                      double* __restrict__ out, long long ld, int nao)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const Tables T = carve(smem);
    const int tid = threadIdx.x;
    const long long p0 = (long long)blockIdx.x * NT + tid;
    const bool valid = p0 < g.npts;
    const long long p = valid ? p0 : 0;
    double x, y, z;
    grid_point(g, valid ? p : g.npts - 1, x, y, z);
    if (tid < 16) T.code[tid] = tid < drv.n ? drv.code[tid] : -1;
    // UB: the channels this instantiation can produce (value; value and first
    // derivatives; all), so that the others are compiled out
    const unsigned chmask = UB == 1u ? 1u : (chmask_in & UB);
    const bool n1 = need_r1(chmask), n2 = need_r2(chmask);
    int w0 = 0, wn = 0, s0 = -SW;
    int last_atom = -1;
    double X = 0.0, Y = 0.0, Z = 0.0, rr = 0.0;
    for (int s = 0; s < B.nshell; ++s) {
        if (s >= s0 + SW) {
            s0 = s;
            stage_shells(B, T, s0);
        }
        const Shell sh = T.sh[s - s0];
        const bool win = sh.nprim <= PW;
        if (win && (sh.prim0 < w0 || sh.prim0 + sh.nprim > w0 + wn)) {
            __syncthreads();
            w0 = sh.prim0;
            wn = B.nprim - w0 < PW ? B.nprim - w0 : PW;
            for (int i = tid; i < 2 * wn; i += NT) T.pa[i] = __ldg(B.prim + 2 * w0 + i);
            __syncthreads();
        }
        if (sh.atom != last_atom) {
            last_atom = sh.atom;
            X = x - __ldg(B.atoms + 4 * sh.atom);
            Y = y - __ldg(B.atoms + 4 * sh.atom + 1);
            Z = z - __ldg(B.atoms + 4 * sh.atom + 2);
            rr = X * X + Y * Y + Z * Z;
        }
        const Radial<double> r = win ? radial64(T.pa, sh.prim0 - w0, sh.nprim, rr, n1, n2)
                                     : radial64(B.prim, sh.prim0, sh.nprim, rr, n1, n2);
        write_shell<SPH>(B, sh, T, X, Y, Z, r, chmask, drv.n, mixed_ref != 0, valid, out, ld, p, nao);
    }
}

template <typename K>
static cudaError_t allow_smem(K kernel, size_t bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <bool SPH, unsigned UB>
static cudaError_t configure_one()
{
    const size_t sm = SPH ? SMEM_SPH : SMEM_CART;
    cudaError_t e = allow_smem(ao_tile_kernel<SPH, UB>, sm);
    if (e == cudaSuccess) e = allow_smem(ao_point_kernel<SPH, UB>, sm);
    return e;
}

static cudaError_t configure()
{
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = configure_one<false, 1u>();
    if (e == cudaSuccess) e = configure_one<false, 0xFu>();
    if (e == cudaSuccess) e = configure_one<false, 0x3FFu>();
    if (e == cudaSuccess) e = configure_one<true, 1u>();
    if (e == cudaSuccess) e = configure_one<true, 0xFu>();
    if (e == cudaSuccess) e = configure_one<true, 0x3FFu>();
    done = e == cudaSuccess;
    return e;
}

template <bool SPH, unsigned UB>
static void launch(bool regular, unsigned nblk, cudaStream_t s, const BasisDev& B, const Grid& g, const DrvList& d,
                   unsigned mask, int mixed_ref, double* out, long long ld, int nao, long long line0, int nzb)
{
    const size_t sm = SPH ? SMEM_SPH : SMEM_CART;
    if (regular)
        ao_tile_kernel<SPH, UB><<<nblk, NT, sm, s>>>(B, g, d, mask, mixed_ref, out, ld, nao, line0, nzb);
    else
        ao_point_kernel<SPH, UB><<<nblk, NT, sm, s>>>(B, g, d, mask, mixed_ref, out, ld, nao);
}

template <bool SPH>
static void launch_mask(bool regular, unsigned nblk, cudaStream_t s, const BasisDev& B, const Grid& g,
                        const DrvList& d, unsigned mask, int mixed_ref, double* out, long long ld, int nao,
                        long long line0, int nzb)
{
    if (mask == 1u)
        launch<SPH, 1u>(regular, nblk, s, B, g, d, mask, mixed_ref, out, ld, nao, line0, nzb);
    else if ((mask & ~0xFu) == 0)
        launch<SPH, 0xFu>(regular, nblk, s, B, g, d, mask, mixed_ref, out, ld, nao, line0, nzb);
    else
        launch<SPH, 0x3FFu>(regular, nblk, s, B, g, d, mask, mixed_ref, out, ld, nao, line0, nzb);
}

}  // namespace ao
}  // namespace okg

using namespace okg;

extern "C" int okg_eval_ao(const okg_basis* b, const okg_grid* grid, int ndrv, const int* h_drv, int exact_mixed,
                           double* d_out, int64_t ld, okg_stream stream)
{
    if (!b || !d_out) return set_error(OKG_ERR_ARG, "okg_eval_ao: NULL basis or output");
    Grid g;
    int st = make_grid(grid, g);
    if (st) return st;
    DrvList d;
    unsigned mask;
    if ((st = make_drv(ndrv, h_drv, d, mask))) return st;
    if (ndrv == 0 || g.npts == 0) return OKG_OK;
    if (ld < g.npts) return set_error(OKG_ERR_ARG, "okg_eval_ao: ld < npts");
    cudaError_t e = ao::configure();
    if (e != cudaSuccess) return cuda_status(e, "okg_eval_ao: shared memory attribute");
    cudaStream_t s = (cudaStream_t)stream;
    const bool sph = b->dev.spherical != 0;
    long long nblk, line0 = 0;
    int nzb = 1;
    if (g.regular) {
        // the grid lines (fixed x, y) holding points [offset, offset + npts)
        line0 = g.offset / g.nz;
        const long long line1 = (g.offset + g.npts - 1) / g.nz;
        const long long nlg = (line1 - line0 + ao::LINES) / ao::LINES;
        nzb = (g.nz + ao::ZB - 1) / ao::ZB;
        nblk = nlg * nzb;
    } else {
        nblk = (g.npts + ao::NT - 1) / ao::NT;
    }
    if (nblk > 0x7FFFFFFFll) return set_error(OKG_ERR_UNSUPPORTED, "okg_eval_ao: grid too large");
    if (sph)
        ao::launch_mask<true>(g.regular != 0, (unsigned)nblk, s, b->dev, g, d, mask, !exact_mixed, d_out, ld,
                              b->nao_out, line0, nzb);
    else
        ao::launch_mask<false>(g.regular != 0, (unsigned)nblk, s, b->dev, g, d, mask, !exact_mixed, d_out, ld,
                               b->nao_out, line0, nzb);
    return cuda_status(cudaGetLastError(), "okg_eval_ao launch");
}
