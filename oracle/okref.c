/*
 * okref.c -- CPU oracle for orbkit's grid path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference algorithm, used by the tests, the smoke
 * check and the CPU-baseline leg of the benchmark as the checker.  It is never
 * part of the product path.  Loop order and floating-point operation order follow
 * the reference so that, compiled without FMA contraction (-ffp-contract=off),
 * its results are bit-identical to the reference's own extension:
 *
 *   okref_ipow / okref_xyz       orbkit/c_support.c:8-26
 *   okref_get_ao_xyz             orbkit/c_support.c:28-175  (drv 0..9, including the
 *                                reference's formula for the mixed derivatives 7-9)
 *   okref_ao_norm                orbkit/c_support.c:177-195
 *   lcreator (static)            orbkit/c_grid-based.c:9-79
 *   okref_aocreator              orbkit/cy_core.pyx:51-78
 *   okref_mocreator              orbkit/cy_core.pyx:82-101
 *   okref_slice_rho              orbkit/core.py:179-304 (slice_rho: AO -> 'N' factor ->
 *                                cartesian2spherical (core.py:135-176) -> MO -> rho, d rho)
 *   okref_rho_threads            the same per slice, slices spread over POSIX threads
 *                                (the reference spreads them over processes,
 *                                core.py:524-537)
 *   okref_aooverlap              orbkit/cy_overlap.pyx:78-163 with get_overlap / s of
 *                                orbkit/c_non-grid-based.c:9-52 (analytic AO overlap)
 *   okref_mooverlapmatrix        orbkit/cy_overlap.pyx:184-205
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

double okref_ipow(double base, int e)
{
    double result = 1.;
    while (e > 0) {
        if (e & 1) result *= base;
        e >>= 1;
        base *= base;
    }
    return result;
}

double okref_xyz(double x, double y, double z, int lx, int ly, int lz)
{
    return okref_ipow(x, lx) * okref_ipow(y, ly) * okref_ipow(z, lz);
}

static int dfact(int n)
{
    return n <= 0 ? 1 : n * dfact(n - 2);
}

double okref_ao_norm(int l, int m, int n, double alpha, int is_normalized)
{
    if (is_normalized > 0) return 1.0;
    return pow((2. / M_PI), (3. / 4.)) * (pow(2., (l + m + n)) * pow(alpha, ((2. * l + 2. * m + 2. * n + 3.) / 4.)))
         / (pow((dfact(2 * l - 1) * dfact(2 * m - 1) * dfact(2 * n - 1)), 0.5));
}

/* Polynomial factor of a primitive Cartesian Gaussian or of one of its derivatives. */
double okref_get_ao_xyz(double X, double Y, double Z, int lx, int ly, int lz, double a, int drv)
{
    double v = 0.;
    switch (drv) {
    case 0: v = okref_xyz(X, Y, Z, lx, ly, lz); break;
    case 1:
        v = (lx == 0) ? -2 * a * okref_xyz(X, Y, Z, lx + 1, ly, lz)
                      : lx * okref_xyz(X, Y, Z, lx - 1, ly, lz) - 2 * a * okref_xyz(X, Y, Z, lx + 1, ly, lz);
        break;
    case 2:
        v = (ly == 0) ? -2 * a * okref_xyz(X, Y, Z, lx, ly + 1, lz)
                      : ly * okref_xyz(X, Y, Z, lx, ly - 1, lz) - 2 * a * okref_xyz(X, Y, Z, lx, ly + 1, lz);
        break;
    case 3:
        v = (lz == 0) ? -2 * a * okref_xyz(X, Y, Z, lx, ly, lz + 1)
                      : lz * okref_xyz(X, Y, Z, lx, ly, lz - 1) - 2 * a * okref_xyz(X, Y, Z, lx, ly, lz + 1);
        break;
    case 4:
        v = 2 * a * okref_xyz(X, Y, Z, lx, ly, lz) * (2 * a * pow(X, 2) - (2 * lx + 1));
        if (lx >= 2) v += (pow(lx, 2) - lx) * okref_xyz(X, Y, Z, lx - 2, ly, lz);
        break;
    case 5:
        v = 2 * a * okref_xyz(X, Y, Z, lx, ly, lz) * (2 * a * pow(Y, 2) - (2 * ly + 1));
        if (ly >= 2) v += (pow(ly, 2) - ly) * okref_xyz(X, Y, Z, lx, ly - 2, lz);
        break;
    case 6:
        v = 2 * a * okref_xyz(X, Y, Z, lx, ly, lz) * (2 * a * pow(Z, 2) - (2 * lz + 1));
        if (lz >= 2) v += (pow(lz, 2) - lz) * okref_xyz(X, Y, Z, lx, ly, lz - 2);
        break;
    case 7:
        v = 4 * pow(a, 2) * okref_xyz(X, Y, Z, lx + 1, ly + 1, lz);
        if (lx == 0 && ly > 0) v += ly * okref_xyz(X, Y, Z, lx, ly - 1, lz);
        else if (lx > 0 && ly == 0) v += lx * okref_xyz(X, Y, Z, lx - 1, ly, lz);
        else if (lx > 0 && ly > 0) v += lx * ly * okref_xyz(X, Y, Z, lx - 1, ly - 1, lz);
        break;
    case 8:
        v = 4 * pow(a, 2) * okref_xyz(X, Y, Z, lx + 1, ly, lz + 1);
        if (lx == 0 && lz > 0) v += lz * okref_xyz(X, Y, Z, lx, ly, lz - 1);
        else if (lx > 0 && lz == 0) v += lx * okref_xyz(X, Y, Z, lx - 1, ly, lz);
        else if (lx > 0 && lz > 0) v += lx * lz * okref_xyz(X, Y, Z, lx - 1, ly, lz - 1);
        break;
    case 9:
        v = 4 * pow(a, 2) * okref_xyz(X, Y, Z, lx, ly + 1, lz + 1);
        if (ly == 0 && lz > 0) v += lz * okref_xyz(X, Y, Z, lx, ly, lz - 1);
        else if (ly > 0 && lz == 0) v += ly * okref_xyz(X, Y, Z, lx, ly - 1, lz);
        else if (ly > 0 && lz > 0) v += ly * lz * okref_xyz(X, Y, Z, lx, ly - 1, lz - 1);
        break;
    default: v = 0.; break; /* the reference prints a message and returns 0 */
    }
    return v;
}

/* One contracted shell on one atom; writes ao[il*npts + i] for its ao_num rows. */
static void lcreator(double* ao, const int* lxlylz, const double* coeff, const double* at, const double* x,
                     const double* y, const double* z, long npts, int ao_num, int pnum, int drv, int is_normalized)
{
    double* norm = (double*)malloc(sizeof(double) * (size_t)ao_num * (size_t)pnum);
    double* ao_l0 = (double*)malloc(sizeof(double) * (size_t)pnum);
    for (int il = 0; il < ao_num; il++)
        for (int ii = 0; ii < pnum; ii++)
            norm[il * pnum + ii] = okref_ao_norm(lxlylz[3 * il], lxlylz[3 * il + 1], lxlylz[3 * il + 2], coeff[2 * ii],
                                                 is_normalized);
    for (long i = 0; i < npts; i++) {
        double X = x[i] - at[0], Y = y[i] - at[1], Z = z[i] - at[2];
        double rr = X * X + Y * Y + Z * Z;
        for (int ii = 0; ii < pnum; ii++) ao_l0[ii] = coeff[2 * ii + 1] * exp(-coeff[2 * ii] * rr);
        for (int il = 0; il < ao_num; il++) {
            int lx = lxlylz[3 * il], ly = lxlylz[3 * il + 1], lz = lxlylz[3 * il + 2];
            double sum = 0.;
            if (drv == 0) {
                for (int ii = 0; ii < pnum; ii++) sum += norm[il * pnum + ii] * ao_l0[ii];
                sum *= okref_xyz(X, Y, Z, lx, ly, lz);
            } else {
                for (int ii = 0; ii < pnum; ii++)
                    sum += norm[il * pnum + ii] * ao_l0[ii] * okref_get_ao_xyz(X, Y, Z, lx, ly, lz, coeff[2 * ii], drv);
            }
            ao[(long)il * npts + i] = sum;
        }
    }
    free(norm);
    free(ao_l0);
}

/* All shells; ao must hold ncart*npts doubles (overwritten). */
void okref_aocreator(double* ao, const int* lxlylz, const int* assign, const double* coeffs, const int* pnum_list,
                     const double* geo, const int* atom_idx, int nshell, const double* x, const double* y,
                     const double* z, long npts, int drv, int is_normalized)
{
    int c_ao = 0, c_p = 0;
    for (int i = 0; i < nshell; i++) {
        lcreator(ao + (long)c_ao * npts, lxlylz + 3 * c_ao, coeffs + 2 * c_p, geo + 3 * atom_idx[i], x, y, z, npts,
                 assign[i], pnum_list[i], drv, is_normalized);
        c_ao += assign[i];
        c_p += pnum_list[i];
    }
}

/* mo[i,j] = sum_k C[i,k] ao[k,j], accumulated in k order. */
void okref_mocreator(double* mo, const double* ao, const double* C, int nao, int nmo, long npts)
{
    for (int i = 0; i < nmo; i++)
        for (long j = 0; j < npts; j++) {
            double value = 0.0;
            for (int k = 0; k < nao; k++) value += C[(long)i * nao + k] * ao[(long)k * npts + j];
            mo[(long)i * npts + j] = value;
        }
}

/* Basis description shared by the slice routines. */
typedef struct {
    const int* lxlylz;
    const int* assign;
    const double* coeffs;
    const int* pnum;
    const double* geo;
    const int* atom_idx;
    int nshell;
    int ncart;
    int is_normalized;
    const double* renorm; /* per Cartesian AO or NULL */
    int nsph;             /* 0: Cartesian output */
    const int* sph_ptr;   /* nsph+1 offsets into sph_idx/sph_coef */
    const int* sph_idx;   /* Cartesian row of each listed component */
    const double* sph_coef;
    const double* C; /* nmo x nao (nao = nsph or ncart) */
    const double* occ;
    int nmo;
} okref_basis;

/* AO rows (Cartesian or spherical) for one derivative code on npts points. */
static void ao_rows(const okref_basis* b, const double* x, const double* y, const double* z, long npts, int drv,
                    double* cart, double* out)
{
    okref_aocreator(cart, b->lxlylz, b->assign, b->coeffs, b->pnum, b->geo, b->atom_idx, b->nshell, x, y, z, npts,
                    drv, b->is_normalized);
    if (b->renorm)
        for (int k = 0; k < b->ncart; k++)
            for (long j = 0; j < npts; j++) cart[(long)k * npts + j] = cart[(long)k * npts + j] * b->renorm[k];
    if (b->nsph) {
        for (int s = 0; s < b->nsph; s++) {
            double* o = out + (long)s * npts;
            for (long j = 0; j < npts; j++) o[j] = 0.0;
            for (int t = b->sph_ptr[s]; t < b->sph_ptr[s + 1]; t++) {
                const double* c = cart + (long)b->sph_idx[t] * npts;
                double f = b->sph_coef[t];
                for (long j = 0; j < npts; j++) o[j] = o[j] + f * c[j];
            }
        }
    } else if (out != cart) {
        memcpy(out, cart, sizeof(double) * (size_t)b->ncart * (size_t)npts);
    }
}

/* One slice of slice_rho: rho (npts) and delta_rho (ndrv x npts).
 * drv[d] is the derivative code; drv2a/drv2b[d] are the first-derivative codes
 * of the product term for two-letter selectors (0 = none); sq[d] marks the
 * squared form ('xx', 'x2' ...).  Returns 0 or -1 on allocation failure. */
int okref_slice_rho(const okref_basis* b, const double* x, const double* y, const double* z, long npts, int ndrv,
                    const int* drv, const int* drv2a, const int* drv2b, const int* sq, double* rho, double* drho,
                    double* mo_norm)
{
    int nao = b->nsph ? b->nsph : b->ncart;
    double* cart = (double*)malloc(sizeof(double) * (size_t)b->ncart * (size_t)npts);
    double* ao = b->nsph ? (double*)malloc(sizeof(double) * (size_t)nao * (size_t)npts) : cart;
    double* mo = (double*)malloc(sizeof(double) * (size_t)b->nmo * (size_t)npts);
    double* dmo = (double*)malloc(sizeof(double) * (size_t)b->nmo * (size_t)npts);
    double* m0 = (double*)malloc(sizeof(double) * (size_t)b->nmo * (size_t)npts);
    double* m1 = (double*)malloc(sizeof(double) * (size_t)b->nmo * (size_t)npts);
    if (!cart || !ao || !mo || !dmo || !m0 || !m1) {
        free(cart); if (b->nsph) free(ao); free(mo); free(dmo); free(m0); free(m1);
        return -1;
    }
    ao_rows(b, x, y, z, npts, 0, cart, ao);
    okref_mocreator(mo, ao, b->C, nao, b->nmo, npts);
    for (long j = 0; j < npts; j++) rho[j] = 0.0;
    for (int i = 0; i < b->nmo; i++) {
        const double* m = mo + (long)i * npts;
        double s = 0.0;
        for (long j = 0; j < npts; j++) {
            rho[j] = rho[j] + b->occ[i] * (m[j] * m[j]);
            s += m[j] * m[j];
        }
        if (mo_norm) mo_norm[i] += s;
    }
    for (int d = 0; d < ndrv; d++) {
        double* dr = drho + (long)d * npts;
        for (long j = 0; j < npts; j++) dr[j] = 0.0;
        ao_rows(b, x, y, z, npts, drv[d], cart, ao);
        okref_mocreator(dmo, ao, b->C, nao, b->nmo, npts);
        int two = drv2a[d] != 0;
        if (two) {
            ao_rows(b, x, y, z, npts, drv2a[d], cart, ao);
            okref_mocreator(m0, ao, b->C, nao, b->nmo, npts);
            if (!sq[d]) {
                ao_rows(b, x, y, z, npts, drv2b[d], cart, ao);
                okref_mocreator(m1, ao, b->C, nao, b->nmo, npts);
            }
        }
        for (int i = 0; i < b->nmo; i++) {
            double o2 = b->occ[i] * 2;
            const double* dm = dmo + (long)i * npts;
            const double* m = mo + (long)i * npts;
            const double* a0 = m0 + (long)i * npts;
            const double* a1 = m1 + (long)i * npts;
            for (long j = 0; j < npts; j++) {
                dr[j] = dr[j] + (o2 * dm[j]) * m[j];
                if (two) dr[j] = dr[j] + o2 * (sq[d] ? a0[j] * a0[j] : a0[j] * a1[j]);
            }
        }
    }
    free(cart); if (b->nsph) free(ao); free(mo); free(dmo); free(m0); free(m1);
    return 0;
}

typedef struct {
    const okref_basis* b;
    const double *x, *y, *z;
    long npts, slice;
    int ndrv;
    const int *drv, *drv2a, *drv2b, *sq;
    double *rho, *drho;
    long next;
    int err;
    pthread_mutex_t lock;
} okref_job;

static void* worker(void* arg)
{
    okref_job* J = (okref_job*)arg;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        long s0 = J->next;
        J->next += J->slice;
        pthread_mutex_unlock(&J->lock);
        if (s0 >= J->npts) break;
        long n = J->npts - s0 < J->slice ? J->npts - s0 : J->slice;
        double* tmp = (double*)malloc(sizeof(double) * (size_t)(J->ndrv > 0 ? J->ndrv : 1) * (size_t)n);
        if (!tmp) { J->err = -1; break; }
        if (okref_slice_rho(J->b, J->x + s0, J->y + s0, J->z + s0, n, J->ndrv, J->drv, J->drv2a, J->drv2b, J->sq,
                            J->rho + s0, tmp, NULL))
            J->err = -1;
        for (int d = 0; d < J->ndrv; d++) memcpy(J->drho + (long)d * J->npts + s0, tmp + (long)d * n, sizeof(double) * n);
        free(tmp);
    }
    return NULL;
}

/* rho / delta_rho over npts points in slices of `slice` points on `nthreads` threads. */
int okref_rho_threads(const okref_basis* b, const double* x, const double* y, const double* z, long npts, int ndrv,
                      const int* drv, const int* drv2a, const int* drv2b, const int* sq, double* rho, double* drho,
                      long slice, int nthreads)
{
    okref_job J;
    J.b = b; J.x = x; J.y = y; J.z = z; J.npts = npts; J.slice = slice > 0 ? slice : 1;
    J.ndrv = ndrv; J.drv = drv; J.drv2a = drv2a; J.drv2b = drv2b; J.sq = sq; J.rho = rho; J.drho = drho;
    J.next = 0; J.err = 0;
    pthread_mutex_init(&J.lock, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    int started = 0;
    for (int t = 0; t < nthreads; t++)
        if (pthread_create(&th[t], NULL, worker, &J) == 0) started++; else break;
    if (started == 0) worker(&J);
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&J.lock);
    return J.err;
}

/* ------------------------------------------------------------------ AO overlap
 * 1D overlap factor s(a, b) along axis i of primitives at RA (exponent al) and
 * RB (exponent be): the recursion orbkit uses (orbkit/c_non-grid-based.c:33-52,
 * after M. Ho and J. M. Hernandez-Perez, Mathematica Journal 14 (2012)). */
static double ov_s(int i, int a, int b, const double* RA, const double* RB, double al, double be)
{
    if (b > 0) return ov_s(i, a + 1, b - 1, RA, RB, al, be) + (RA[i] - RB[i]) * ov_s(i, a, b - 1, RA, RB, al, be);
    if (a == 0) return 1.;
    const double xpa = -(RA[i] - (al * RA[i] + be * RB[i]) / (al + be));
    if (a == 1) return xpa;
    return xpa * ov_s(i, a - 1, 0, RA, RB, al, be) + ((a - 1) / (2. * (al + be))) * ov_s(i, a - 2, 0, RA, RB, al, be);
}

/* Primitive overlap (orbkit/c_non-grid-based.c:9-31). */
static double ov_prim(const double* RA, const int* la, double al, const double* RB, const int* lb, double be)
{
    double rr = 0;
    for (int i = 0; i < 3; i++) rr += (RA[i] - RB[i]) * (RA[i] - RB[i]);
    double ov = exp(-((al * be) / (al + be)) * rr) * pow(M_PI / (al + be), 3. / 2.);
    for (int i = 0; i < 3; i++) ov *= ov_s(i, la[i], lb[i], RA, RB, al, be);
    return ov;
}

/* cy_overlap.aooverlap (orbkit/cy_overlap.pyx:78-163): aoom (ncart x ncart, zeroed
 * by the caller) over the flattened (shell, row, primitive) list, bra outer, ket
 * inner; drv 1..3 differentiates the ket along x, y, z. */
void okref_aooverlap(double* aoom, const double* geo_a, const double* geo_b, const int* lxlylz_a,
                     const int* lxlylz_b, const int* assign, const double* coeffs, const int* pnum, const int* atoms,
                     int nshell, int drv, int is_normalized)
{
    int nidx = 0, ncart = 0;
    for (int s = 0; s < nshell; s++) {
        nidx += assign[s] * pnum[s];
        ncart += assign[s];
    }
    int* row = (int*)malloc(sizeof(int) * (size_t)nidx);
    int* prm = (int*)malloc(sizeof(int) * (size_t)nidx);
    int* atm = (int*)malloc(sizeof(int) * (size_t)nidx);
    double* nrm = (double*)malloc(sizeof(double) * (size_t)nidx);
    int c = 0, c_ao = 0, c_p = 0;
    for (int s = 0; s < nshell; s++) {
        for (int r = 0; r < assign[s]; r++)
            for (int q = 0; q < pnum[s]; q++) {
                const int* l = lxlylz_a + 3 * (c_ao + r);
                nrm[c] = okref_ao_norm(l[0], l[1], l[2], coeffs[2 * (c_p + q)], is_normalized);
                row[c] = c_ao + r;
                prm[c] = c_p + q;
                atm[c] = atoms[s];
                c++;
            }
        c_ao += assign[s];
        c_p += pnum[s];
    }
    for (int i = 0; i < nidx; i++)
        for (int j = 0; j < nidx; j++) {
            const double* RA = geo_a + 3 * atm[i];
            const double* RB = geo_b + 3 * atm[j];
            const int* la = lxlylz_a + 3 * row[i];
            int lb[3] = {lxlylz_b[3 * row[j]], lxlylz_b[3 * row[j] + 1], lxlylz_b[3 * row[j] + 2]};
            const double al = coeffs[2 * prm[i]], be = coeffs[2 * prm[j]];
            const double ci = coeffs[2 * prm[i] + 1], cj = coeffs[2 * prm[j] + 1];
            double* out = aoom + (long)row[i] * ncart + row[j];
            if (drv <= 0) {
                *out += ci * cj * nrm[i] * nrm[j] * ov_prim(RA, la, al, RB, lb, be);
                continue;
            }
            const int d = drv - 1, l0 = lb[d];
            if (l0 > 0) {
                lb[d] = l0 - 1;
                *out += l0 * ci * cj * nrm[i] * nrm[j] * ov_prim(RA, la, al, RB, lb, be);
            }
            lb[d] = l0 + 1;
            *out += (-2 * be) * ci * cj * nrm[i] * nrm[j] * ov_prim(RA, la, al, RB, lb, be);
        }
    free(row);
    free(prm);
    free(atm);
    free(nrm);
    (void)ncart;
}

/* cy_overlap.mooverlapmatrix (orbkit/cy_overlap.pyx:184-205): moom[i,j] =
 * sum_k sum_l a[i,k] b[j,l] S[k,l], k outer, l inner. */
void okref_mooverlapmatrix(double* moom, const double* A, const double* B, const double* S, int nmo_a, int nmo_b,
                           int nao, int mao)
{
    for (int i = 0; i < nmo_a; i++)
        for (int j = 0; j < nmo_b; j++) {
            double t = 0.0;
            for (int k = 0; k < nao; k++)
                for (int l = 0; l < mao; l++) t += A[(long)i * nao + k] * B[(long)j * mao + l] * S[(long)k * mao + l];
            moom[(long)i * nmo_b + j] = t;
        }
}
