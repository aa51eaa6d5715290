// Internal device structures and shell-evaluation templates shared by the
// orbkit_gb300 kernels.  Math follows orbkit's c_lcreator / get_ao_xyz /
// ao_norm (orbkit/c_grid-based.c:9-79, orbkit/c_support.c:8-195), reorganised
// for the GPU: per (shell, point) the primitive exponentials are computed once
// and reduced to three radial sums
//     R0 = sum_p w_p e_p,  R1 = sum_p w_p a_p e_p,  R2 = sum_p w_p a_p^2 e_p
// (w_p = contraction coefficient x alpha-dependent primitive norm, e_p = exp(-a_p r^2));
// every Cartesian component and every derivative up to second order is then a
// short polynomial in X, Y, Z times these sums.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/orbkit_gb300.h"

#define OKG_MAX_L 4
#define OKG_MAX_NCART 15  // (L+1)(L+2)/2 at L = 4

namespace okg {

// ---------------------------------------------------------------- tables
// Canonical (Molden) order of the Cartesian components per L
// (the order of orbkit/tools.py:117-135); a shell may list its components in
// another order, comp_row maps canonical index -> listed row.
__host__ __device__ constexpr int ncanon(int L) { return (L + 1) * (L + 2) / 2; }

__host__ __device__ constexpr int canon_l(int L, int j, int axis)
{
    // rows: (lx, ly, lz)
    constexpr int t0[1][3] = {{0, 0, 0}};
    constexpr int t1[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    constexpr int t2[6][3] = {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
    constexpr int t3[10][3] = {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {1, 2, 0}, {2, 1, 0},
                               {2, 0, 1}, {1, 0, 2}, {0, 1, 2}, {0, 2, 1}, {1, 1, 1}};
    constexpr int t4[15][3] = {{4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1}, {1, 0, 3},
                               {0, 1, 3}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}};
    return L == 0 ? t0[j][axis] : L == 1 ? t1[j][axis] : L == 2 ? t2[j][axis] : L == 3 ? t3[j][axis] : t4[j][axis];
}

struct Shell {
    int atom;   // atom index (into BasisDev::atoms)
    int L;      // angular momentum
    int nprim;  // primitives
    int prim0;  // first primitive
    int cart0;  // first listed Cartesian row (global)
    int ncart;  // listed components
    int comp0;  // offset of this shell's ncanon(L) entries in comp_row / comp_g
    int out0;   // first output row (Cartesian: cart0, spherical: first spherical row)
    int nout;   // output rows (ncart or number of spherical functions)
    int sph0;   // first spherical row's index into sph_ptr (spherical bases)
    int mcol;   // mixed path (records of BasisDev::mshells): first column of this shell inside its chunk
    int mchunk; // mixed path (records of BasisDev::mshells): index of the chunk holding this shell
};

// Per-primitive data of the mixed path: alpha*log2(e) in FP64 (the exponent
// argument stays FP64) and the weights w, w*alpha in FP32.
struct PrimMx {
    double a2;
    float w;
    float wa;
};

struct BasisDev {
    const double* atoms;     // natom x 4 (x, y, z, unused)
    const Shell* shells;     // nshell
    const double* prim;      // nprim x 2 : alpha, w (w includes the alpha-dependent norm)
    const float* prim32;     // nprim x 4 : alpha*log2(e) (hi, lo), w (hi, lo) for the mixed path
    const int* prim_atom;    // nprim : atom of each primitive
    const int* comp_row;     // per shell canonical component -> listed row within shell, or -1
    const double* comp_g;    // per shell canonical component -> angular norm factor x 'N'
    const int* sph_ptr;      // nsph + 1
    const int* sph_cidx;     // canonical component index within the shell
    const double* sph_coef;  // coefficient x global factor
    const int4* chunks;      // nchunk x {first shell, end shell, first Cartesian row, end row}
    const PrimMx* prim_mx;   // nprim (mixed path)
    const double* prim_adj;  // nprim x 2 : dw/dalpha, w/c (the alpha-dependent norm) for the adjoint
    const double2* prim_cusp;  // nprim (mixed path): {alpha, w} in FP64, in the order of prim_mx (ascending alpha per shell)
    const int* atom_shell_ptr; // natom + 1: shells of atom a are atom_shells[atom_shell_ptr[a] .. atom_shell_ptr[a+1])
    const int* atom_shells;    // nshell
    const Shell* mshells;    // nshell: the shells in the mixed path's column order (okg_basis_set_mixed_order)
    const int4* mchunks;     // nmchunk x {first, end index into mshells, used columns, 0} (<= OKG_MKC columns)
    const int* mcol_cart;    // nmchunk x OKG_MKC: listed Cartesian row feeding each column, or -1
    const double* mcol_g;    // nmchunk x OKG_MKC: angular norm of each column (0 where unused)
    int natom, nshell, nprim, ncart, nsph, spherical;
    int max_nprim, nchunk, nmchunk;
};

// Mixed path: chunks of whole shells with at most OKG_MKC canonical columns
// (one 64-byte swizzle row of BF16 values).
#define OKG_MKC 32

// Shells are grouped into chunks of at most KC listed Cartesian rows; the fused
// kernels stage one chunk of AO values in shared memory at a time.
#define OKG_KC 32

// Grid: vector grid (x, y, z arrays) or regular grid (x slowest, z fastest).
struct Grid {
    const double* x;
    const double* y;
    const double* z;
    long long npts;    // points in this call
    long long offset;  // first point (regular grids: flattened index)
    int nx, ny, nz;
    int regular;
};

__device__ __forceinline__ void grid_point(const Grid& g, long long p, double& x, double& y, double& z)
{
    if (g.regular) {
        long long q = p + g.offset;
        long long nyz = (long long)g.ny * g.nz;
        int i = (int)(q / nyz);
        long long r = q - (long long)i * nyz;
        int j = (int)(r / g.nz);
        int k = (int)(r - (long long)j * g.nz);
        x = __ldg(g.x + i);
        y = __ldg(g.y + j);
        z = __ldg(g.z + k);
    } else {
        x = __ldg(g.x + p);
        y = __ldg(g.y + p);
        z = __ldg(g.z + p);
    }
}

// Channels: 0 value, 1..3 d/dx d/dy d/dz, 4..6 d2/dx2 d2/dy2 d2/dz2, 7..9 d2/dxdy dxdz dydz
// (orbkit's drv codes, orbkit/c_support.c:28-50).
enum { CH_VAL = 1u, CH_GRAD = 0xEu, CH_HESS_D = 0x70u, CH_HESS_O = 0x380u };

// Radial sums of one shell at one point, FP64.
template <typename T>
struct Radial {
    T R0, R1, R2;
};

__device__ __forceinline__ Radial<double> radial64(const double* __restrict__ prim, int p0, int np, double rr,
                                                   bool need1, bool need2)
{
    Radial<double> r{0.0, 0.0, 0.0};
    for (int q = 0; q < np; ++q) {
        const double a = prim[2 * (p0 + q)];
        if (a * rr > 746.0) continue;  // exp(-a rr) is 0 in double: the primitive adds exactly 0
        const double w = prim[2 * (p0 + q) + 1];
        const double e = w * exp(-a * rr);
        r.R0 += e;
        if (need1) r.R1 += a * e;
        if (need2) r.R2 += a * a * e;
    }
    return r;
}

// Value of channel ch for the canonical component (a, b, c) given powers
// px[i] = X^i (i <= L + 2) etc.  mixed_ref selects orbkit's formula for the
// mixed second derivatives (c_support.c:121-168), which omits the -2 alpha
// cross terms of the exact derivative; the exact form is used otherwise.
template <int a, int b, int c, typename T>
__device__ __forceinline__ T channel_poly(int ch, const T* px, const T* py, const T* pz, const Radial<T>& r,
                                          bool mixed_ref)
{
    // 1D factors for the first and second derivative along one axis
    auto d1 = [&](const T* p, int n) -> T {  // n X^{n-1} R0 - 2 X^{n+1} R1
        T v = T(-2) * p[n + 1] * r.R1;
        if (n > 0) v += T(n) * p[n - 1] * r.R0;
        return v;
    };
    auto d2 = [&](const T* p, int n) -> T {  // n(n-1) X^{n-2} R0 - 2(2n+1) X^n R1 + 4 X^{n+2} R2
        T v = T(4) * p[n + 2] * r.R2 - T(2 * (2 * n + 1)) * p[n] * r.R1;
        if (n > 1) v += T(n * (n - 1)) * p[n - 2] * r.R0;
        return v;
    };
    auto mixed = [&](const T* pu, int nu, const T* pv, int nv) -> T {
        T v = T(4) * pu[nu + 1] * pv[nv + 1] * r.R2;
        if (mixed_ref) {
            if (nu > 0 || nv > 0) {
                T q = T(1);
                if (nu > 0) q *= T(nu) * pu[nu - 1];
                if (nv > 0) q *= T(nv) * pv[nv - 1];
                v += q * r.R0;
            }
        } else {
            T t = pu[nu + 1] * (nv > 0 ? T(nv) * pv[nv - 1] : T(0));
            if (nu > 0) t += T(nu) * pu[nu - 1] * pv[nv + 1];
            v -= T(2) * t * r.R1;
            if (nu > 0 && nv > 0) v += T(nu * nv) * pu[nu - 1] * pv[nv - 1] * r.R0;
        }
        return v;
    };
    switch (ch) {
    case 0: return px[a] * py[b] * pz[c] * r.R0;
    case 1: return d1(px, a) * py[b] * pz[c];
    case 2: return px[a] * d1(py, b) * pz[c];
    case 3: return px[a] * py[b] * d1(pz, c);
    case 4: return d2(px, a) * py[b] * pz[c];
    case 5: return px[a] * d2(py, b) * pz[c];
    case 6: return px[a] * py[b] * d2(pz, c);
    case 7: return mixed(px, a, py, b) * pz[c];
    case 8: return mixed(px, a, pz, c) * py[b];
    default: return mixed(py, b, pz, c) * px[a];
    }
}

// Evaluate all canonical components of an L shell for the channels in chmask
// and hand each value to sink(channel, canonical index, value).  The angular
// norm factor is *not* applied (the sink multiplies by comp_g).
template <int L, typename T, typename Sink>
__device__ __forceinline__ void shell_eval(T X, T Y, T Z, const Radial<T>& r, unsigned chmask, bool mixed_ref,
                                           Sink&& sink)
{
    T px[L + 3], py[L + 3], pz[L + 3];
    px[0] = py[0] = pz[0] = T(1);
#pragma unroll
    for (int i = 1; i < L + 3; ++i) {
        px[i] = px[i - 1] * X;
        py[i] = py[i - 1] * Y;
        pz[i] = pz[i - 1] * Z;
    }
#pragma unroll
    for (int ch = 0; ch < 10; ++ch) {
        if (!(chmask & (1u << ch))) continue;
        [&]<int... J>(std::integer_sequence<int, J...>) {
            (sink(ch, J,
                  channel_poly<canon_l(L, J, 0), canon_l(L, J, 1), canon_l(L, J, 2), T>(ch, px, py, pz, r, mixed_ref)),
             ...);
        }(std::make_integer_sequence<int, ncanon(L)>{});
    }
}

template <typename T, typename Sink>
__device__ __forceinline__ void shell_eval_L(int L, T X, T Y, T Z, const Radial<T>& r, unsigned chmask,
                                             bool mixed_ref, Sink&& sink)
{
    switch (L) {
    case 0: shell_eval<0>(X, Y, Z, r, chmask, mixed_ref, sink); break;
    case 1: shell_eval<1>(X, Y, Z, r, chmask, mixed_ref, sink); break;
    case 2: shell_eval<2>(X, Y, Z, r, chmask, mixed_ref, sink); break;
    case 3: shell_eval<3>(X, Y, Z, r, chmask, mixed_ref, sink); break;
    default: shell_eval<4>(X, Y, Z, r, chmask, mixed_ref, sink); break;
    }
}

// which radial sums a channel mask needs
__host__ __device__ inline bool need_r1(unsigned m) { return (m & ~1u) != 0; }
__host__ __device__ inline bool need_r2(unsigned m) { return (m & (CH_HESS_D | CH_HESS_O)) != 0; }

}  // namespace okg

// Host-side helpers shared by the translation units (okg_api.cu).
struct okg_basis {
    okg::BasisDev dev;
    void* dev_block;  // single device allocation holding every table
    size_t dev_bytes;
    int* h_shell_L;   // unused (kept zero)
    int* prim_L;      // device: angular momentum of each primitive's shell
    int is_normalized;
    int natom, nshell, nprim, ncart, nao_out, max_l;
    int l_hist[OKG_MAX_L + 1];
    int device;
    int ncomp;                 // entries of comp_row / comp_g
    mutable int mixed_locked;  // a mixed plan or evaluation used the basis: its column order is fixed
};

namespace okg {
int set_error(int status, const char* msg);
int cuda_status(cudaError_t e, const char* where);

// Requested derivative codes of a call (orbkit's drv codes 0..9).
struct DrvList {
    int n;
    int code[10];
};

// okg_grid -> Grid with the checks every grid entry point makes.
inline int make_grid(const okg_grid* gr, Grid& g)
{
    if (!gr) return set_error(OKG_ERR_ARG, "grid is NULL");
    g.x = gr->d_x;
    g.y = gr->d_y;
    g.z = gr->d_z;
    g.npts = gr->npts;
    g.offset = gr->offset;
    g.nx = gr->nx;
    g.ny = gr->ny;
    g.nz = gr->nz;
    g.regular = gr->regular;
    if (g.npts < 0 || !g.x || !g.y || !g.z) return set_error(OKG_ERR_ARG, "grid: NULL coordinates or npts < 0");
    if (g.regular) {
        if (g.nx <= 0 || g.ny <= 0 || g.nz <= 0 || g.offset < 0 ||
            g.offset + g.npts > (long long)g.nx * g.ny * g.nz)
            return set_error(OKG_ERR_ARG, "grid: regular grid range outside Nx*Ny*Nz");
    }
    return OKG_OK;
}

// Derivative codes -> DrvList and the mask of channels they need.
inline int make_drv(int ndrv, const int* h_drv, DrvList& d, unsigned& mask)
{
    if (ndrv < 0 || ndrv > 10 || (ndrv > 0 && !h_drv)) return set_error(OKG_ERR_ARG, "drv: 0..10 codes required");
    d.n = ndrv;
    mask = 0;
    for (int i = 0; i < 10; ++i) d.code[i] = 0;
    for (int i = 0; i < ndrv; ++i) {
        if (h_drv[i] < 0 || h_drv[i] > 9) return set_error(OKG_ERR_DRV, "drv: code outside 0..9");
        d.code[i] = h_drv[i];
        mask |= 1u << h_drv[i];
    }
    return OKG_OK;
}
}  // namespace okg
