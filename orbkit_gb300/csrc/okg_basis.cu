// Basis packing, parameter upload and status reporting for liborbkit_gb300.
//
// okg_basis_create flattens orbkit's AO description (the arrays produced by
// AOClass getters, orbkit/orbitals.py:336-385) into one device block of tables:
// shells, canonical-component maps with the angular norm factors
// 1/sqrt((2l-1)!!(2m-1)!!(2n-1)!!) times the optional per-AO 'N' factor
// (orbkit/c_support.c:177-195, orbkit/core.py:98-100), the spherical transform
// (orbkit/core.py:135-176) and the shell chunks used by the fused kernels.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "okg_internal.cuh"

namespace okg {

static thread_local std::string g_last_error;

int set_error(int status, const char* msg)
{
    g_last_error = msg ? msg : "";
    return status;
}

int cuda_status(cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return OKG_OK;
    // consume the runtime's last-error state of this (non-sticky) error, so that a later
    // cudaGetLastError() after a good launch does not report it again
    (void)cudaGetLastError();
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    g_last_error = m;
    return e == cudaErrorMemoryAllocation ? OKG_ERR_ALLOC : OKG_ERR_CUDA;
}

static int dfact(int n) { return n <= 0 ? 1 : n * dfact(n - 2); }

// Primitive weights w = c * (2/pi)^(3/4) 2^L alpha^((2L+3)/4) (or c when the
// contractions are pre-normalised) and the split single-precision copies used by
// the mixed path.
__global__ void prim_weights_kernel(const double* __restrict__ prim_in, const int* __restrict__ prim_L, int nprim,
                                    int is_normalized, double* __restrict__ prim_out, float* __restrict__ prim32,
                                    PrimMx* __restrict__ prim_mx, double* __restrict__ prim_adj,
                                    double2* __restrict__ prim_cusp)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nprim) return;
    const double a = prim_in[2 * i];
    const double c = prim_in[2 * i + 1];
    const int L = prim_L[i];
    double w = c, nrm = 1.0, dw = 0.0;
    if (!is_normalized) {
        nrm = pow(2.0 / M_PI, 0.75) * (pow(2.0, (double)L) * pow(a, (2.0 * L + 3.0) / 4.0));
        w = c * nrm;
        dw = w * (2.0 * L + 3.0) / (4.0 * a);  // d w / d alpha
    }
    prim_adj[2 * i] = dw;
    prim_adj[2 * i + 1] = nrm;
    prim_out[2 * i] = a;
    prim_out[2 * i + 1] = w;
    // mixed path: alpha * log2(e) and w as float hi + lo pairs
    const double al = a * 1.4426950408889634;
    const float ah = (float)al;
    const float wh = (float)w;
    prim32[4 * i + 0] = ah;
    prim32[4 * i + 1] = (float)(al - (double)ah);
    prim32[4 * i + 2] = wh;
    prim32[4 * i + 3] = (float)(w - (double)wh);
    PrimMx m;
    m.a2 = al;
    m.w = wh;
    m.wa = (float)(w * a);
    prim_mx[i] = m;
    prim_cusp[i] = make_double2(a, w);
}

// Mixed path: order each shell's primitives by ascending exponent, so that a
// tile keeps a prefix of them when screening (the radial sums do not depend on
// the order).  One thread per shell, insertion sort (a handful of primitives).
// The FP64 {alpha, w} copy used for the cusp points of the mixed path is sorted
// along (same permutation).
__global__ void sort_prim_mx_kernel(const Shell* __restrict__ shells, int nshell, PrimMx* __restrict__ prim_mx,
                                    double2* __restrict__ prim_cusp)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nshell) return;
    const int p0 = shells[s].prim0, np = shells[s].nprim;
    for (int i = 1; i < np; ++i) {
        const PrimMx v = prim_mx[p0 + i];
        const double2 c = prim_cusp[p0 + i];
        int j = i - 1;
        while (j >= 0 && prim_mx[p0 + j].a2 > v.a2) {
            prim_mx[p0 + j + 1] = prim_mx[p0 + j];
            prim_cusp[p0 + j + 1] = prim_cusp[p0 + j];
            --j;
        }
        prim_mx[p0 + j + 1] = v;
        prim_cusp[p0 + j + 1] = c;
    }
}

__global__ void atoms_kernel(const double* __restrict__ geo, int natom, double* __restrict__ atoms)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= natom) return;
    atoms[4 * i + 0] = geo[3 * i + 0];
    atoms[4 * i + 1] = geo[3 * i + 1];
    atoms[4 * i + 2] = geo[3 * i + 2];
    atoms[4 * i + 3] = 0.0;
}

}  // namespace okg

using namespace okg;

extern "C" const char* okg_status_string(int s)
{
    switch (s) {
    case OKG_OK: return "ok";
    case OKG_ERR_ARG: return "invalid argument";
    case OKG_ERR_L: return "unsupported angular momentum";
    case OKG_ERR_DRV: return "invalid derivative code";
    case OKG_ERR_CUDA: return "CUDA error";
    case OKG_ERR_ALLOC: return "allocation failed";
    case OKG_ERR_TIMEOUT: return "device wait timed out";
    case OKG_ERR_UNSUPPORTED: return "unsupported shape";
    case OKG_ERR_DEVICE: return "no usable device";
    default: return "unknown status";
    }
}

extern "C" const char* okg_last_error(void) { return g_last_error.c_str(); }

extern "C" int okg_version(void) { return 100; }

namespace {
struct Layout {
    size_t off = 0;
    size_t take(size_t bytes)
    {
        size_t o = (off + 255) & ~(size_t)255;
        off = o + bytes;
        return o;
    }
};

// Mixed-path column layout for a shell order: whole shells, in that order, packed
// into chunks of at most OKG_MKC canonical columns; per chunk column, the listed
// Cartesian row it feeds (or -1) and its angular norm.  At most one chunk per shell.
struct MixedLayout {
    std::vector<Shell> mshells;
    std::vector<int4> mchunks;
    std::vector<int> mcol_cart;
    std::vector<double> mcol_g;
};

MixedLayout mixed_layout(const std::vector<Shell>& shells, const std::vector<int>& comp_row,
                         const std::vector<double>& comp_g, const int* order)
{
    MixedLayout m;
    const int n = (int)shells.size();
    int s0 = 0, col = 0;
    for (int i = 0; i <= n; ++i) {
        const int nk = i < n ? ncanon(shells[order ? order[i] : i].L) : 0;
        if (i == n || col + nk > OKG_MKC) {
            m.mchunks.push_back(make_int4(s0, i, col, 0));
            const size_t base = m.mcol_cart.size();
            m.mcol_cart.resize(base + OKG_MKC, -1);
            m.mcol_g.resize(base + OKG_MKC, 0.0);
            for (int t = s0; t < i; ++t) {
                const Shell& sh = m.mshells[t];
                for (int q = 0; q < ncanon(sh.L); ++q) {
                    const int r = comp_row[sh.comp0 + q];
                    if (r >= 0) {
                        m.mcol_cart[base + sh.mcol + q] = sh.cart0 + r;
                        m.mcol_g[base + sh.mcol + q] = comp_g[sh.comp0 + q];
                    }
                }
            }
            s0 = i;
            col = 0;
        }
        if (i < n) {
            Shell sh = shells[order ? order[i] : i];
            sh.mcol = col;
            sh.mchunk = (int)m.mchunks.size();
            m.mshells.push_back(sh);
            col += nk;
        }
    }
    return m;
}

// Upload a mixed layout into the basis block (capacity: one chunk per shell).
cudaError_t upload_mixed(okg_basis* b, const MixedLayout& m)
{
    BasisDev& d = b->dev;
    cudaError_t e = cudaMemcpy((void*)d.mshells, m.mshells.data(), sizeof(Shell) * m.mshells.size(),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy((void*)d.mchunks, m.mchunks.data(), sizeof(int4) * m.mchunks.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy((void*)d.mcol_cart, m.mcol_cart.data(), sizeof(int) * m.mcol_cart.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy((void*)d.mcol_g, m.mcol_g.data(), sizeof(double) * m.mcol_g.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) d.nmchunk = (int)m.mchunks.size();
    return e;
}
}  // namespace

extern "C" int okg_basis_create(int natom, int nshell, const int* h_shell_atom, const int* h_shell_ncart,
                                const int* h_shell_nprim, const int* h_lxlylz, int is_normalized,
                                const double* h_renorm, int nsph, const int* h_sph_ptr, const int* h_sph_cart,
                                const double* h_sph_coef, okg_basis** out)
{
    if (!out) return set_error(OKG_ERR_ARG, "okg_basis_create: out is NULL");
    *out = nullptr;
    if (natom <= 0 || nshell <= 0 || !h_shell_atom || !h_shell_ncart || !h_shell_nprim || !h_lxlylz)
        return set_error(OKG_ERR_ARG, "okg_basis_create: empty basis or NULL array");
    if (nsph < 0 || (nsph > 0 && (!h_sph_ptr || !h_sph_cart || !h_sph_coef)))
        return set_error(OKG_ERR_ARG, "okg_basis_create: spherical transform arrays missing");

    std::vector<Shell> shells(nshell);
    std::vector<int> comp_row;
    std::vector<double> comp_g;
    std::vector<int> prim_L;
    std::vector<int> prim_atom;  // atom of each primitive (the AO kernel's per-axis tables)
    int ncart = 0, nprim = 0, max_np = 0, max_l = 0;
    int l_hist[OKG_MAX_L + 1] = {0};
    for (int s = 0; s < nshell; ++s) {
        const int nc = h_shell_ncart[s], np = h_shell_nprim[s], at = h_shell_atom[s];
        if (nc <= 0 || np <= 0 || at < 0 || at >= natom)
            return set_error(OKG_ERR_ARG, "okg_basis_create: shell with no components/primitives or bad atom index");
        const int* l0 = h_lxlylz + 3 * ncart;
        const int L = l0[0] + l0[1] + l0[2];
        if (L < 0 || L > OKG_MAX_L) return set_error(OKG_ERR_L, "okg_basis_create: angular momentum above 4");
        Shell& sh = shells[s];
        sh.atom = at;
        sh.L = L;
        sh.nprim = np;
        sh.prim0 = nprim;
        sh.cart0 = ncart;
        sh.ncart = nc;
        sh.comp0 = (int)comp_row.size();
        sh.out0 = ncart;
        sh.nout = nc;
        sh.sph0 = 0;
        const int nk = ncanon(L);
        if (nc > nk) return set_error(OKG_ERR_L, "okg_basis_create: more components than the shell's L allows");
        comp_row.resize(sh.comp0 + nk, -1);
        comp_g.resize(sh.comp0 + nk, 0.0);
        for (int r = 0; r < nc; ++r) {
            const int* lc = h_lxlylz + 3 * (ncart + r);
            if (lc[0] < 0 || lc[1] < 0 || lc[2] < 0 || lc[0] + lc[1] + lc[2] != L)
                return set_error(OKG_ERR_L, "okg_basis_create: components of mixed angular momentum in one shell");
            int j = -1;
            for (int q = 0; q < nk; ++q)
                if (canon_l(L, q, 0) == lc[0] && canon_l(L, q, 1) == lc[1] && canon_l(L, q, 2) == lc[2]) j = q;
            if (j < 0 || comp_row[sh.comp0 + j] >= 0)
                return set_error(OKG_ERR_L, "okg_basis_create: repeated Cartesian component in one shell");
            comp_row[sh.comp0 + j] = r;
            double g = is_normalized ? 1.0 : 1.0 / sqrt((double)(dfact(2 * lc[0] - 1) * dfact(2 * lc[1] - 1) *
                                                                  dfact(2 * lc[2] - 1)));
            if (h_renorm) g *= h_renorm[ncart + r];
            comp_g[sh.comp0 + j] = g;
        }
        for (int q = 0; q < np; ++q) {
            prim_L.push_back(L);
            prim_atom.push_back(at);
        }
        ncart += nc;
        nprim += np;
        max_np = np > max_np ? np : max_np;
        max_l = L > max_l ? L : max_l;
        l_hist[L]++;
    }

    // spherical transform -> (canonical component within shell, coefficient)
    std::vector<int> sph_ptr(1, 0), sph_cidx;
    std::vector<double> sph_coef;
    if (nsph > 0) {
        std::vector<int> row_shell(ncart), row_canon(ncart);
        for (int s = 0; s < nshell; ++s) {
            const Shell& sh = shells[s];
            for (int q = 0; q < ncanon(sh.L); ++q) {
                int r = comp_row[sh.comp0 + q];
                if (r >= 0) {
                    row_shell[sh.cart0 + r] = s;
                    row_canon[sh.cart0 + r] = q;
                }
            }
            shells[s].nout = 0;
        }
        int prev_shell = -1;
        for (int r = 0; r < nsph; ++r) {
            const int t0 = h_sph_ptr[r], t1 = h_sph_ptr[r + 1];
            if (t1 <= t0) return set_error(OKG_ERR_ARG, "okg_basis_create: spherical row without components");
            int s = -1;
            for (int t = t0; t < t1; ++t) {
                const int c = h_sph_cart[t];
                if (c < 0 || c >= ncart) return set_error(OKG_ERR_ARG, "okg_basis_create: spherical component index");
                if (s >= 0 && row_shell[c] != s)
                    return set_error(OKG_ERR_ARG, "okg_basis_create: spherical row mixes shells");
                s = row_shell[c];
                sph_cidx.push_back(row_canon[c]);
                sph_coef.push_back(h_sph_coef[t]);
            }
            sph_ptr.push_back((int)sph_cidx.size());
            if (s != prev_shell) {
                if (shells[s].nout != 0)
                    return set_error(OKG_ERR_ARG, "okg_basis_create: spherical rows of a shell are not contiguous");
                shells[s].out0 = r;
                shells[s].sph0 = r;
                prev_shell = s;
            }
            shells[s].nout++;
        }
    }

    // chunks of whole shells with at most OKG_KC listed rows
    std::vector<int4> chunks;
    {
        int s0 = 0, k0 = 0, k = 0;
        for (int s = 0; s < nshell; ++s) {
            if (k + shells[s].ncart - k0 > OKG_KC) {
                chunks.push_back(make_int4(s0, s, k0, k));
                s0 = s;
                k0 = k;
            }
            k += shells[s].ncart;
        }
        chunks.push_back(make_int4(s0, nshell, k0, k));
    }

    // mixed-path chunks in basis order (okg_basis_set_mixed_order may choose another)
    const MixedLayout mixed = mixed_layout(shells, comp_row, comp_g, nullptr);

    okg_basis* b = (okg_basis*)calloc(1, sizeof(okg_basis));
    if (!b) return set_error(OKG_ERR_ALLOC, "okg_basis_create: host allocation");
    Layout lay;
    const size_t o_atoms = lay.take(sizeof(double) * 4 * natom);
    const size_t o_shells = lay.take(sizeof(Shell) * nshell);
    const size_t o_prim = lay.take(sizeof(double) * 2 * nprim);
    const size_t o_prim32 = lay.take(sizeof(float) * 4 * nprim);
    const size_t o_primL = lay.take(sizeof(int) * nprim);
    const size_t o_patom = lay.take(sizeof(int) * nprim);
    const size_t o_crow = lay.take(sizeof(int) * comp_row.size());
    const size_t o_cg = lay.take(sizeof(double) * comp_g.size());
    const size_t o_sptr = lay.take(sizeof(int) * sph_ptr.size());
    const size_t o_scid = lay.take(sizeof(int) * (sph_cidx.size() + 1));
    const size_t o_scoef = lay.take(sizeof(double) * (sph_coef.size() + 1));
    const size_t o_chunks = lay.take(sizeof(int4) * chunks.size());
    const size_t o_pmx = lay.take(sizeof(PrimMx) * nprim);
    const size_t o_pcusp = lay.take(sizeof(double2) * nprim);
    const size_t o_asp = lay.take(sizeof(int) * (natom + 1));
    const size_t o_ash = lay.take(sizeof(int) * nshell);
    const size_t o_padj = lay.take(sizeof(double) * 2 * nprim);
    const size_t o_msh = lay.take(sizeof(Shell) * nshell);
    const size_t o_mch = lay.take(sizeof(int4) * nshell);
    const size_t o_mcc = lay.take(sizeof(int) * OKG_MKC * nshell);
    const size_t o_mcg = lay.take(sizeof(double) * OKG_MKC * nshell);
    const size_t bytes = lay.take(0);
    char* blk = nullptr;
    cudaError_t e = cudaMalloc((void**)&blk, bytes);
    if (e != cudaSuccess) {
        free(b);
        return cuda_status(e, "okg_basis_create: cudaMalloc");
    }
    e = cudaMemset(blk, 0, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(blk + o_shells, shells.data(), sizeof(Shell) * nshell, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(blk + o_primL, prim_L.data(), sizeof(int) * nprim, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(blk + o_patom, prim_atom.data(), sizeof(int) * nprim, cudaMemcpyHostToDevice);
    // shells of each atom (CSR), for the cusp points of the mixed path
    std::vector<int> atom_shell_ptr(natom + 1, 0), atom_shells(nshell);
    for (int s = 0; s < nshell; ++s) atom_shell_ptr[shells[s].atom + 1]++;
    for (int a = 0; a < natom; ++a) atom_shell_ptr[a + 1] += atom_shell_ptr[a];
    {
        std::vector<int> fill(atom_shell_ptr.begin(), atom_shell_ptr.end() - 1);
        for (int s = 0; s < nshell; ++s) atom_shells[fill[shells[s].atom]++] = s;
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(blk + o_asp, atom_shell_ptr.data(), sizeof(int) * (natom + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(blk + o_ash, atom_shells.data(), sizeof(int) * nshell, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(blk + o_crow, comp_row.data(), sizeof(int) * comp_row.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(blk + o_cg, comp_g.data(), sizeof(double) * comp_g.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(blk + o_sptr, sph_ptr.data(), sizeof(int) * sph_ptr.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !sph_cidx.empty())
        e = cudaMemcpy(blk + o_scid, sph_cidx.data(), sizeof(int) * sph_cidx.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !sph_coef.empty())
        e = cudaMemcpy(blk + o_scoef, sph_coef.data(), sizeof(double) * sph_coef.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(blk + o_chunks, chunks.data(), sizeof(int4) * chunks.size(), cudaMemcpyHostToDevice);
    BasisDev& d = b->dev;
    d.mshells = (const Shell*)(blk + o_msh);
    d.mchunks = (const int4*)(blk + o_mch);
    d.mcol_cart = (const int*)(blk + o_mcc);
    d.mcol_g = (const double*)(blk + o_mcg);
    if (e == cudaSuccess) e = upload_mixed(b, mixed);
    if (e != cudaSuccess) {
        cudaFree(blk);
        free(b);
        return cuda_status(e, "okg_basis_create: upload");
    }
    b->dev_block = blk;
    b->dev_bytes = bytes;
    d.atoms = (const double*)(blk + o_atoms);
    d.shells = (const Shell*)(blk + o_shells);
    d.prim = (const double*)(blk + o_prim);
    d.prim32 = (const float*)(blk + o_prim32);
    d.prim_atom = (const int*)(blk + o_patom);
    d.comp_row = (const int*)(blk + o_crow);
    d.comp_g = (const double*)(blk + o_cg);
    d.sph_ptr = (const int*)(blk + o_sptr);
    d.sph_cidx = (const int*)(blk + o_scid);
    d.sph_coef = (const double*)(blk + o_scoef);
    d.chunks = (const int4*)(blk + o_chunks);
    d.prim_mx = (const PrimMx*)(blk + o_pmx);
    d.prim_cusp = (const double2*)(blk + o_pcusp);
    d.atom_shell_ptr = (const int*)(blk + o_asp);
    d.atom_shells = (const int*)(blk + o_ash);
    d.prim_adj = (const double*)(blk + o_padj);
    d.natom = natom;
    d.nshell = nshell;
    d.nprim = nprim;
    d.ncart = ncart;
    d.nsph = nsph;
    d.spherical = nsph > 0;
    d.max_nprim = max_np;
    d.nchunk = (int)chunks.size();
    b->h_shell_L = nullptr;
    b->natom = natom;
    b->nshell = nshell;
    b->nprim = nprim;
    b->ncart = ncart;
    b->nao_out = nsph > 0 ? nsph : ncart;
    b->max_l = max_l;
    for (int l = 0; l <= OKG_MAX_L; ++l) b->l_hist[l] = l_hist[l];
    b->is_normalized = is_normalized ? 1 : 0;
    b->prim_L = (int*)(blk + o_primL);
    b->ncomp = (int)comp_row.size();
    b->mixed_locked = 0;
    cudaGetDevice(&b->device);
    *out = b;
    return OKG_OK;
}

extern "C" int okg_basis_set_mixed_order(okg_basis* b, const int* h_order)
{
    if (!b || !h_order) return set_error(OKG_ERR_ARG, "okg_basis_set_mixed_order: NULL argument");
    if (b->mixed_locked)
        return set_error(OKG_ERR_ARG, "okg_basis_set_mixed_order: a mixed plan or evaluation already uses the basis");
    const int n = b->nshell;
    std::vector<char> seen(n, 0);
    for (int i = 0; i < n; ++i) {
        if (h_order[i] < 0 || h_order[i] >= n || seen[h_order[i]])
            return set_error(OKG_ERR_ARG, "okg_basis_set_mixed_order: order is not a permutation of the shells");
        seen[h_order[i]] = 1;
    }
    std::vector<Shell> shells(n);
    std::vector<int> comp_row(b->ncomp);
    std::vector<double> comp_g(b->ncomp);
    cudaError_t e = cudaMemcpy(shells.data(), b->dev.shells, sizeof(Shell) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(comp_row.data(), b->dev.comp_row, sizeof(int) * b->ncomp, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(comp_g.data(), b->dev.comp_g, sizeof(double) * b->ncomp, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = upload_mixed(b, mixed_layout(shells, comp_row, comp_g, h_order));
    return cuda_status(e, "okg_basis_set_mixed_order");
}

extern "C" int okg_basis_destroy(okg_basis* b)
{
    if (!b) return OKG_OK;
    cudaError_t e = cudaFree(b->dev_block);
    free(b);
    return cuda_status(e, "okg_basis_destroy");
}

extern "C" int okg_basis_info(const okg_basis* b, int* ncart, int* nao, int* nshell, int* nprim, int* natom)
{
    if (!b) return set_error(OKG_ERR_ARG, "okg_basis_info: NULL basis");
    if (ncart) *ncart = b->ncart;
    if (nao) *nao = b->nao_out;
    if (nshell) *nshell = b->nshell;
    if (nprim) *nprim = b->nprim;
    if (natom) *natom = b->natom;
    return OKG_OK;
}

extern "C" int okg_basis_set_params(okg_basis* b, const double* d_geo, const double* d_prim, okg_stream stream)
{
    if (!b || !d_geo || !d_prim) return set_error(OKG_ERR_ARG, "okg_basis_set_params: NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    atoms_kernel<<<(b->natom + 127) / 128, 128, 0, st>>>(d_geo, b->natom, (double*)b->dev.atoms);
    prim_weights_kernel<<<(b->nprim + 127) / 128, 128, 0, st>>>(d_prim, b->prim_L, b->nprim, b->is_normalized,
                                                                 (double*)b->dev.prim, (float*)b->dev.prim32,
                                                                 (PrimMx*)b->dev.prim_mx, (double*)b->dev.prim_adj,
                                                                 (double2*)b->dev.prim_cusp);
    sort_prim_mx_kernel<<<(b->nshell + 127) / 128, 128, 0, st>>>(b->dev.shells, b->nshell, (PrimMx*)b->dev.prim_mx,
                                                                 (double2*)b->dev.prim_cusp);
    return cuda_status(cudaGetLastError(), "okg_basis_set_params");
}
