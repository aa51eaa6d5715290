// Analytic overlap of contracted Cartesian Gaussians between a bra basis at one
// geometry and a ket basis at another, with an optional first derivative of the ket
// and optional ket exponents: orbkit's get_ao_overlap
// (orbkit/analytical_integrals.py:37-116) over cy_overlap.aooverlap
// (orbkit/cy_overlap.pyx:78-163) and get_overlap (orbkit/c_non-grid-based.c:9-52).
//
// Per call, a table holds what a primitive pair shares across all component pairs of
// its two shells (p, the prefactor, P - A; ov_pairs_kernel).  Then one thread per
// output Cartesian pair (I, J).  It walks the primitives of I (outer)
// and of J (inner), which is the order orbkit's flattened primitive loop adds them
// to aoom[I, J].  The 1D factors are evaluated with orbkit's operations and
// rounding (IEEE divisions, no FMA contraction): the two terms of a derivative can
// cancel to a small fraction of their size, and only this keeps such elements
// within 1e-12 of orbkit's.  The factors common to all terms of a primitive pair,
// exp(-mu R^2) and (pi/p)^(3/2), use one reciprocal of p and a square root (a few
// units in the last place from orbkit's exp/pow values).  The 1D factors follow the recursion of
// M. Ho and J. M. Hernandez-Perez, "Evaluation of Gaussian Molecular Integrals",
// Mathematica Journal 14 (2012), doi:10.3888/tmj.14-3, that orbkit uses:
//   s(0,0) = 1,  s(1,0) = P - A,
//   s(a,0) = (P - A) s(a-1,0) + (a-1)/(2p) s(a-2,0),
//   s(a,b) = s(a+1,b-1) + (A - B) s(a,b-1),
// evaluated bottom-up in a small table instead of recursively (same values).
//
// A derivative d/dx_d of the ket (drv = d + 1) replaces its 1D factor along d by
// l s(l_a, l_b - 1) - 2 beta s(l_a, l_b + 1) (only the second term when l_b = 0),
// the two terms added to the element separately as orbkit does.
//
// The plan holds the basis tables on the device: per listed Cartesian row its
// primitive range, atom and packed exponents (bra from ao_spec, ket optionally
// overridden), the primitive (alpha, c) pairs and the primitive norms
// ao_norm(l, m, n, alpha) of orbkit/c_support.c:177-188 per (row, primitive),
// computed on the host once with the same formula.  The per-AO 'N' factor and the
// spherical transform (orbkit/analytical_integrals.py:109-116, 118-182) are applied
// by a second kernel: out[r, s] = sum_a sum_b k_a k_b (N_a N_b S[a, b]).
#include <math.h>

#include <algorithm>
#include <vector>

#include "okg_internal.cuh"

#define OKG_OV_MAXV 24  // longest vertical recursion: max l_bra + max l_ket + 2
#define OV_PAIR_TABLE_MAX (2ull << 30)  // bytes of the primitive-pair table a plan may hold

namespace okg {

struct OvRow {
    int prim0;  // first primitive (into prim)
    int nprim;
    int atom;
    int rp0;    // first (row, primitive) norm
    int la;     // bra exponents packed lx | ly << 8 | lz << 16
    int lb;     // ket exponents, same packing
};

__device__ __forceinline__ int lcomp(int packed, int d) { return (packed >> (8 * d)) & 0xff; }

// s(la, lb) along one axis (and, for the derivative axis, s(la, lb - 1) and
// s(la, lb + 1)).  v holds s(a, k) for a >= la after transfer round k.
__device__ __forceinline__ void os_axis(double xpa, double ab, double p, int la, int lb, bool deriv, double* v,
                                        double& s0, double& sm, double& sp)
{
    const int top = la + lb + (deriv ? 1 : 0);
    v[0] = 1.0;
    if (top >= 1) v[1] = xpa;
    for (int a = 2; a <= top; ++a)
        v[a] = __dadd_rn(__dmul_rn(xpa, v[a - 1]), __dmul_rn((double)(a - 1) / (2.0 * p), v[a - 2]));
    s0 = v[la];
    sm = 0.0;
    const int rounds = lb + (deriv ? 1 : 0);
    for (int k = 1; k <= rounds; ++k) {
        if (deriv && k == lb) sm = v[la];  // s(la, lb - 1) is v[la] after round lb - 1
        for (int a = la; a <= top - k; ++a) v[a] = __dadd_rn(v[a + 1], __dmul_rn(ab, v[a]));
        if (k == lb) s0 = v[la];
    }
    sp = v[la];
}

// Quantities of a primitive pair (bra primitive i at its atom in geo_a, ket primitive j
// at its atom in geo_b) shared by every Cartesian component pair of the two shells:
// p = alpha + beta, pref = exp(-mu R^2) (pi/p)^(3/2) (0 where the exponential
// underflows) and P - A per axis.  Evaluated once per call into a table of
// nprim x nprim entries when the plan holds one, with the same operations as the
// element kernel's own evaluation.
struct alignas(16) OvPair {
    double pref, p, xpa[3], pad;
};

__global__ void ov_pairs_kernel(int nprim, const double2* __restrict__ prim, const int* __restrict__ prim_atom,
                                const double* __restrict__ geo_a, const double* __restrict__ geo_b,
                                OvPair* __restrict__ pairs)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nprim || j >= nprim) return;
    const double al = prim[i].x, be = prim[j].x;
    double A[3], B[3];
    double rr = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        A[d] = geo_a[3 * prim_atom[i] + d];
        B[d] = geo_b[3 * prim_atom[j] + d];
        const double ab = A[d] - B[d];
        rr = fma(ab, ab, rr);
    }
    OvPair e;
    const double inv_p = 1.0 / (al + be);
    const double arg = al * be * inv_p * rr;
    e.p = al + be;
    if (arg > 746.0) {
        e.pref = 0.0;  // exp(-arg) is 0 in double
    } else {
        const double t = M_PI * inv_p;
        e.pref = exp(-arg) * t * sqrt(t);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double P = __dadd_rn(__dmul_rn(al, A[d]), __dmul_rn(be, B[d])) / e.p;
        e.xpa[d] = -(A[d] - P);
    }
    e.pad = 0.0;
    pairs[(long long)i * nprim + j] = e;
}

// A warp computes 32 elements of one bra row I.  Its kets are consecutive in the
// plan's ket order (sorted by primitive count, then exponents), so the lanes run
// the same primitive loops and recursion lengths; a primitive pair is skipped only
// when exp(-mu R^2) underflows for every lane (it contributes exactly 0 to the
// others as well).
template <bool TABLE>
__global__ void __launch_bounds__(256) ao_overlap_kernel(int nrow, const OvRow* __restrict__ rows,
                                                         const int* __restrict__ ket_order,
                                                         const double2* __restrict__ prim,
                                                         const double* __restrict__ pnorm,
                                                         const double* __restrict__ geo_a,
                                                         const double* __restrict__ geo_b,
                                                         const OvPair* __restrict__ pairs, int nprim, int drv,
                                                         double* __restrict__ out, long long ld)
{
    const int Jo = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = blockIdx.y * blockDim.y + threadIdx.y;
    if (I >= nrow || Jo >= nrow) return;
    const int J = ket_order[Jo];
    const OvRow ri = rows[I], rj = rows[J];
    double A[3], B[3], AB[3];
    double rr = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        A[d] = geo_a[3 * ri.atom + d];
        B[d] = geo_b[3 * rj.atom + d];
        AB[d] = A[d] - B[d];
        rr = fma(AB[d], AB[d], rr);
    }
    const int dd = drv - 1;  // derivative axis or -1
    double v[OKG_OV_MAXV];
    double acc = 0.0;
    for (int ip = 0; ip < ri.nprim; ++ip) {
        const double2 pa = prim[ri.prim0 + ip];
        const double na = pnorm[ri.rp0 + ip];
        for (int jp = 0; jp < rj.nprim; ++jp) {
            const double2 pb = prim[rj.prim0 + jp];
            const double nb = pnorm[rj.rp0 + jp];
            const double al = pa.x, be = pb.x;
            double pref, p, xpa_t[3];
            if (TABLE) {
                const double2* e = reinterpret_cast<const double2*>(pairs + (long long)(ri.prim0 + ip) * nprim +
                                                                   rj.prim0 + jp);
                const double2 e0 = e[0], e1 = e[1], e2 = e[2];
                pref = e0.x;
                p = e0.y;
                xpa_t[0] = e1.x;
                xpa_t[1] = e1.y;
                xpa_t[2] = e2.x;
                if (__all_sync(__activemask(), pref == 0.0)) continue;  // the pair adds exactly 0
            } else {
                const double inv_p = 1.0 / (al + be);
                const double arg = al * be * inv_p * rr;
                if (__all_sync(__activemask(), arg > 746.0)) continue;  // exp(-arg) is 0 in double: adds exactly 0
                const double eab = exp(-arg);
                const double t = M_PI * inv_p;
                pref = eab * t * sqrt(t);
                p = al + be;
            }
            // product of the 1D factors of the non-derivative axes, in axis order;
            // along the derivative axis the two shifted factors are kept apart
            double s_plain = pref, s_minus = pref, s_plus = pref;
            int lbd = 0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double xpa;
                if (TABLE) {
                    xpa = xpa_t[d];
                } else {
                    const double P = __dadd_rn(__dmul_rn(al, A[d]), __dmul_rn(be, B[d])) / p;
                    xpa = -(A[d] - P);
                }
                const int la = lcomp(ri.la, d), lb = lcomp(rj.lb, d);
                const bool deriv = (d == dd);
                double s0, sm, sp;
                os_axis(xpa, AB[d], p, la, lb, deriv, v, s0, sm, sp);
                if (deriv) {
                    lbd = lb;
                    s_minus = __dmul_rn(s_minus, sm);
                    s_plus = __dmul_rn(s_plus, sp);
                    s_plain = __dmul_rn(s_plain, s0);
                } else {
                    s_plain = __dmul_rn(s_plain, s0);
                    s_minus = __dmul_rn(s_minus, s0);
                    s_plus = __dmul_rn(s_plus, s0);
                }
            }
            const double cc = __dmul_rn(pa.y, pb.y);
            if (dd < 0) {
                acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(__dmul_rn(cc, na), nb), s_plain));
            } else {
                if (lbd > 0) {
                    const double t = __dmul_rn(__dmul_rn(__dmul_rn((double)lbd * pa.y, pb.y), na), nb);
                    acc = __dadd_rn(acc, __dmul_rn(t, s_minus));
                }
                const double t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(-2.0 * be, pa.y), pb.y), na), nb);
                acc = __dadd_rn(acc, __dmul_rn(t, s_plus));
            }
        }
    }
    out[(long long)I * ld + J] = acc;
}

// out[r, s] = sum_{a in r} sum_{b in s} (k_a k_b) (N_a N_b S[a, b]); for a Cartesian
// output (nsph = 0) the rows are the Cartesian rows with k = 1.
__global__ void aoom_transform_kernel(int nout, const int* __restrict__ ptr, const int* __restrict__ cart,
                                      const double* __restrict__ coef, const double* __restrict__ renorm,
                                      const double* __restrict__ S, long long lds, double* __restrict__ out,
                                      long long ld)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (r >= nout || s >= nout) return;
    double acc = 0.0;
    for (int i = ptr[r]; i < ptr[r + 1]; ++i) {
        const int a = cart[i];
        const double ka = coef[i];
        const double na = renorm ? renorm[a] : 1.0;
        for (int j = ptr[s]; j < ptr[s + 1]; ++j) {
            const int b = cart[j];
            double sab = S[(long long)a * lds + b];
            if (renorm) sab = __dmul_rn(__dmul_rn(na, renorm[b]), sab);
            acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(ka, coef[j]), sab));
        }
    }
    out[(long long)r * ld + s] = acc;
}

}  // namespace okg

using namespace okg;

struct okg_overlap_plan {
    int* ket_order = nullptr;  // kets sorted by (primitive count, exponents): the kernel's column order
    int* prim_atom = nullptr;  // atom of every primitive
    OvPair* pairs = nullptr;   // nprim x nprim primitive-pair table (NULL above OV_PAIR_TABLE_MAX bytes)
    int natom, nshell, ncart, nprim, nout;
    int max_la;
    int spherical, has_renorm;
    std::vector<OvRow> h_rows;
    std::vector<int> h_lxa;  // ncart x 3 (bra)
    OvRow* rows = nullptr;
    double2* prim = nullptr;
    double* pnorm = nullptr;
    double* renorm = nullptr;
    int* tptr = nullptr;    // transform rows (nout + 1)
    int* tcart = nullptr;
    double* tcoef = nullptr;
    double* work = nullptr; // ncart x ncart Cartesian matrix before the transform
    int max_lb;             // of the current ket exponents
    int device;
};

static double ov_dfact(int n) { return n <= 0 ? 1.0 : n * ov_dfact(n - 2); }

// orbkit/c_support.c:177-188 (ao_norm), evaluated on the host as orbkit does.
static double ov_ao_norm(int l, int m, int n, double alpha, int is_normalized)
{
    if (is_normalized > 0) return 1.0;
    return pow(2. / M_PI, 3. / 4.) * (pow(2., l + m + n) * pow(alpha, (2. * l + 2. * m + 2. * n + 3.) / 4.)) /
           pow(ov_dfact(2 * l - 1) * ov_dfact(2 * m - 1) * ov_dfact(2 * n - 1), 0.5);
}

static int ov_pack(const int* l) { return l[0] | (l[1] << 8) | (l[2] << 16); }

// Kets sorted by (primitive count, packed ket exponents, row): rows a warp handles
// together then run the same loops.
static std::vector<int> ov_ket_order(const std::vector<OvRow>& rows)
{
    std::vector<int> o(rows.size());
    for (size_t i = 0; i < o.size(); ++i) o[i] = (int)i;
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) {
        if (rows[a].nprim != rows[b].nprim) return rows[a].nprim < rows[b].nprim;
        return rows[a].lb < rows[b].lb;
    });
    return o;
}

static void ov_free(okg_overlap_plan* p)
{
    if (!p) return;
    cudaFree(p->rows);
    cudaFree(p->prim);
    cudaFree(p->pnorm);
    cudaFree(p->renorm);
    cudaFree(p->tptr);
    cudaFree(p->tcart);
    cudaFree(p->tcoef);
    cudaFree(p->work);
    cudaFree(p->ket_order);
    cudaFree(p->prim_atom);
    cudaFree(p->pairs);
    delete p;
}

template <class T>
static int ov_upload(T** dst, const T* src, size_t n, const char* what)
{
    if (n == 0) return OKG_OK;
    cudaError_t e = cudaMalloc((void**)dst, n * sizeof(T));
    if (e != cudaSuccess) return cuda_status(e, what);
    return cuda_status(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice), what);
}

extern "C" int okg_overlap_plan_create(int natom, int nshell, const int* h_shell_atom, const int* h_shell_ncart,
                                       const int* h_shell_nprim, const int* h_lxlylz, int is_normalized,
                                       const double* h_prim, const double* h_renorm, int nsph, const int* h_sph_ptr,
                                       const int* h_sph_cart, const double* h_sph_coef, okg_overlap_plan** out)
{
    if (!out) return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: out is NULL");
    *out = nullptr;
    if (natom <= 0 || nshell <= 0 || !h_shell_atom || !h_shell_ncart || !h_shell_nprim || !h_lxlylz || !h_prim)
        return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: empty basis or NULL array");
    if (nsph < 0 || (nsph > 0 && (!h_sph_ptr || !h_sph_cart || !h_sph_coef)))
        return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: spherical transform arrays missing");
    okg_overlap_plan* P = new okg_overlap_plan();
    P->natom = natom;
    P->nshell = nshell;
    int ncart = 0, nprim = 0, nrp = 0, max_l = 0;
    for (int s = 0; s < nshell; ++s) {
        const int nc = h_shell_ncart[s], np = h_shell_nprim[s], at = h_shell_atom[s];
        if (nc <= 0 || np <= 0 || at < 0 || at >= natom) {
            delete P;
            return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: shell with no components/primitives or bad atom");
        }
        for (int r = 0; r < nc; ++r) {
            const int* l = h_lxlylz + 3 * (ncart + r);
            for (int d = 0; d < 3; ++d) {
                if (l[d] < 0 || l[d] > 64) {
                    delete P;
                    return set_error(OKG_ERR_L, "okg_overlap_plan_create: Cartesian exponent outside 0..64");
                }
                max_l = l[d] > max_l ? l[d] : max_l;
            }
            OvRow row;
            row.prim0 = nprim;
            row.nprim = np;
            row.atom = at;
            row.rp0 = nrp;
            row.la = row.lb = ov_pack(l);
            P->h_rows.push_back(row);
            P->h_lxa.insert(P->h_lxa.end(), l, l + 3);
            nrp += np;
        }
        ncart += nc;
        nprim += np;
    }
    if (2 * max_l + 2 > OKG_OV_MAXV - 1) {
        delete P;
        return set_error(OKG_ERR_L, "okg_overlap_plan_create: Cartesian exponent too large for the overlap tables");
    }
    std::vector<double2> prim(nprim);
    for (int i = 0; i < nprim; ++i) prim[i] = make_double2(h_prim[2 * i], h_prim[2 * i + 1]);
    std::vector<double> pnorm(nrp);
    for (int r = 0; r < ncart; ++r) {
        const OvRow& row = P->h_rows[r];
        const int* l = &P->h_lxa[3 * r];
        for (int q = 0; q < row.nprim; ++q)
            pnorm[row.rp0 + q] = ov_ao_norm(l[0], l[1], l[2], prim[row.prim0 + q].x, is_normalized);
    }
    // transform rows: spherical rows from the tables, else one Cartesian row each
    std::vector<int> tptr, tcart;
    std::vector<double> tcoef;
    if (nsph > 0) {
        if (h_sph_ptr[0] != 0) {
            delete P;
            return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: sph_ptr[0] must be 0");
        }
        for (int r = 0; r <= nsph; ++r) tptr.push_back(h_sph_ptr[r]);
        for (int r = 0; r < nsph; ++r)
            if (h_sph_ptr[r + 1] < h_sph_ptr[r]) {
                delete P;
                return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: sph_ptr not ascending");
            }
        for (int i = 0; i < h_sph_ptr[nsph]; ++i) {
            if (h_sph_cart[i] < 0 || h_sph_cart[i] >= ncart) {
                delete P;
                return set_error(OKG_ERR_ARG, "okg_overlap_plan_create: spherical component outside the Cartesian rows");
            }
            tcart.push_back(h_sph_cart[i]);
            tcoef.push_back(h_sph_coef[i]);
        }
    } else {
        for (int r = 0; r <= ncart; ++r) tptr.push_back(r);
        for (int r = 0; r < ncart; ++r) {
            tcart.push_back(r);
            tcoef.push_back(1.0);
        }
    }
    cudaGetDevice(&P->device);
    P->ncart = ncart;
    P->nprim = nprim;
    P->nout = nsph > 0 ? nsph : ncart;
    P->spherical = nsph > 0;
    P->has_renorm = h_renorm != nullptr;
    P->max_la = max_l;
    P->max_lb = max_l;
    int st = OKG_OK;
    if ((st = ov_upload(&P->rows, P->h_rows.data(), P->h_rows.size(), "okg_overlap_plan_create")) ||
        (st = ov_upload(&P->prim, prim.data(), prim.size(), "okg_overlap_plan_create")) ||
        (st = ov_upload(&P->pnorm, pnorm.data(), pnorm.size(), "okg_overlap_plan_create")) ||
        (h_renorm && (st = ov_upload(&P->renorm, h_renorm, (size_t)ncart, "okg_overlap_plan_create"))) ||
        (st = ov_upload(&P->tptr, tptr.data(), tptr.size(), "okg_overlap_plan_create")) ||
        (st = ov_upload(&P->tcart, tcart.data(), tcart.size(), "okg_overlap_plan_create")) ||
        (st = ov_upload(&P->tcoef, tcoef.data(), tcoef.size(), "okg_overlap_plan_create")) ||
        (st = ov_upload(&P->ket_order, ov_ket_order(P->h_rows).data(), (size_t)ncart, "okg_overlap_plan_create"))) {
        ov_free(P);
        return st;
    }
    cudaError_t e = cudaMalloc((void**)&P->work, (size_t)ncart * ncart * sizeof(double));
    if (e != cudaSuccess) {
        ov_free(P);
        return cuda_status(e, "okg_overlap_plan_create: workspace");
    }
    // primitive-pair table (geometry-dependent, filled by every okg_ao_overlap call)
    const size_t pair_bytes = (size_t)nprim * nprim * sizeof(OvPair);
    if (pair_bytes <= OV_PAIR_TABLE_MAX) {
        std::vector<int> prim_atom;
        prim_atom.reserve(nprim);
        for (int sh = 0; sh < nshell; ++sh)
            for (int q = 0; q < h_shell_nprim[sh]; ++q) prim_atom.push_back(h_shell_atom[sh]);
        if ((st = ov_upload(&P->prim_atom, prim_atom.data(), prim_atom.size(), "okg_overlap_plan_create"))) {
            ov_free(P);
            return st;
        }
        e = cudaMalloc((void**)&P->pairs, pair_bytes);
        if (e != cudaSuccess) {
            ov_free(P);
            return cuda_status(e, "okg_overlap_plan_create: primitive-pair table");
        }
    }
    *out = P;
    return OKG_OK;
}

extern "C" int okg_overlap_plan_destroy(okg_overlap_plan* plan)
{
    ov_free(plan);
    return OKG_OK;
}

extern "C" int okg_overlap_plan_info(const okg_overlap_plan* plan, int* ncart, int* nao)
{
    if (!plan) return set_error(OKG_ERR_ARG, "okg_overlap_plan_info: NULL plan");
    if (ncart) *ncart = plan->ncart;
    if (nao) *nao = plan->nout;
    return OKG_OK;
}

extern "C" int okg_overlap_plan_set_ket(okg_overlap_plan* plan, const int* h_lxlylz_b)
{
    if (!plan) return set_error(OKG_ERR_ARG, "okg_overlap_plan_set_ket: NULL plan");
    int max_lb = 0;
    for (int r = 0; r < plan->ncart; ++r) {
        const int* l = h_lxlylz_b ? h_lxlylz_b + 3 * r : &plan->h_lxa[3 * r];
        for (int d = 0; d < 3; ++d) {
            if (l[d] < 0 || l[d] > 64) return set_error(OKG_ERR_L, "okg_overlap_plan_set_ket: exponent outside 0..64");
            max_lb = l[d] > max_lb ? l[d] : max_lb;
        }
    }
    if (plan->max_la + max_lb + 2 > OKG_OV_MAXV - 1)
        return set_error(OKG_ERR_L, "okg_overlap_plan_set_ket: exponents too large for the overlap tables");
    for (int r = 0; r < plan->ncart; ++r) {
        const int* l = h_lxlylz_b ? h_lxlylz_b + 3 * r : &plan->h_lxa[3 * r];
        plan->h_rows[r].lb = ov_pack(l);
    }
    plan->max_lb = max_lb;
    int st = cuda_status(cudaMemcpy(plan->rows, plan->h_rows.data(), plan->h_rows.size() * sizeof(OvRow),
                                    cudaMemcpyHostToDevice),
                         "okg_overlap_plan_set_ket");
    if (st) return st;
    const std::vector<int> order = ov_ket_order(plan->h_rows);
    return cuda_status(cudaMemcpy(plan->ket_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice),
                       "okg_overlap_plan_set_ket");
}

extern "C" int okg_ao_overlap(okg_overlap_plan* plan, const double* d_geo_a, const double* d_geo_b, int drv,
                              int raw, double* d_out, int64_t ld, okg_stream stream)
{
    if (!plan || !d_geo_a || !d_geo_b || !d_out)
        return set_error(OKG_ERR_ARG, "okg_ao_overlap: NULL plan, geometry or output");
    if (drv < 0 || drv > 3)
        return set_error(OKG_ERR_DRV, "okg_ao_overlap: only drv 0 (none) and 1..3 (d/dx, d/dy, d/dz) are supported");
    const int nout = raw ? plan->ncart : plan->nout;
    if (ld < nout) return set_error(OKG_ERR_ARG, "okg_ao_overlap: ld smaller than the matrix");
    cudaStream_t st = (cudaStream_t)stream;
    const bool direct = raw || (!plan->spherical && !plan->has_renorm);
    double* S = direct ? d_out : plan->work;
    const long long lds = direct ? ld : plan->ncart;
    const dim3 blk(32, 8);
    const dim3 grd((plan->ncart + 31) / 32, (plan->ncart + 7) / 8);
    if (plan->pairs) {
        const dim3 gpp((plan->nprim + 31) / 32, (plan->nprim + 7) / 8);
        ov_pairs_kernel<<<gpp, blk, 0, st>>>(plan->nprim, plan->prim, plan->prim_atom, d_geo_a, d_geo_b, plan->pairs);
        ao_overlap_kernel<true><<<grd, blk, 0, st>>>(plan->ncart, plan->rows, plan->ket_order, plan->prim,
                                                    plan->pnorm, d_geo_a, d_geo_b, plan->pairs, plan->nprim, drv,
                                                    S, lds);
    } else {
        ao_overlap_kernel<false><<<grd, blk, 0, st>>>(plan->ncart, plan->rows, plan->ket_order, plan->prim,
                                                     plan->pnorm, d_geo_a, d_geo_b, nullptr, 0, drv, S, lds);
    }
    int s = cuda_status(cudaGetLastError(), "okg_ao_overlap launch");
    if (s || direct) return s;
    const dim3 tblk(16, 16);
    const dim3 grt((plan->nout + 15) / 16, (plan->nout + 15) / 16);
    aoom_transform_kernel<<<grt, tblk, 0, st>>>(plan->nout, plan->tptr, plan->tcart, plan->tcoef, plan->renorm, S,
                                               lds, d_out, ld);
    return cuda_status(cudaGetLastError(), "okg_ao_overlap transform launch");
}
