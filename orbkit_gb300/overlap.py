"""Analytic overlap of contracted Cartesian Gaussians (input preparation, CPU).

Not part of the grid path: it prepares inputs.  The synthetic workloads use it
to normalise contractions and to Loewdin-orthonormalise MO coefficients, which is
what orbkit's ``analytical_integrals.get_ao_overlap`` (analytical_integrals.py:37-116,
cy_overlap.pyx:78-163, c_non-grid-based.c:9-52) is used for.  Conventions match
orbkit: primitive normalisation ``ao_norm`` (c_support.c:177-188), the optional
per-AO factor ``ao_spec[0]['N']`` and the spherical transform of ``tools.cart2sph``.

The 1D factors use the Obara-Saika recurrences (Obara & Saika, J. Chem. Phys. 84,
3963 (1986)), vectorised over all primitive pairs of one (la, lb) class.  Pairs
whose Gaussian product prefactor exp(-mu R^2) is below exp(-46) (about 1e-20)
are skipped.
"""
import numpy

from .tools import doublefactorial, get_cart2sph

_SCREEN = 46.0


def ao_norm(l, m, n, alpha, is_normalized=0):
    """Primitive normalisation (2/pi)^(3/4) 2^L alpha^((2L+3)/4) / sqrt((2l-1)!!(2m-1)!!(2n-1)!!)."""
    if is_normalized:
        return numpy.ones_like(numpy.asarray(alpha, dtype=numpy.float64))
    L = l + m + n
    return ((2.0 / numpy.pi) ** 0.75 * (2.0 ** L * numpy.asarray(alpha, dtype=numpy.float64) ** ((2.0 * L + 3.0) / 4.0))
            / numpy.sqrt(float(doublefactorial(2 * l - 1) * doublefactorial(2 * m - 1) * doublefactorial(2 * n - 1))))


def _os_1d(xpa, xpb, oo2p, la, lb):
    """1D overlap factors S[a][b] for a<=la, b<=lb (each an array over pairs)."""
    S = [[None] * (lb + 1) for _ in range(la + 1)]
    one = numpy.ones_like(xpa)
    S[0][0] = one
    for a in range(1, la + 1):
        v = xpa * S[a - 1][0]
        if a >= 2:
            v = v + (a - 1) * oo2p * S[a - 2][0]
        S[a][0] = v
    for b in range(1, lb + 1):
        for a in range(0, la + 1):
            v = xpb * S[a][b - 1]
            if a >= 1:
                v = v + a * oo2p * S[a - 1][b - 1]
            if b >= 2:
                v = v + (b - 1) * oo2p * S[a][b - 2]
            S[a][b] = v
    return S


def cartesian_overlap(geo, ao_spec):
    """(NAOcart, NAOcart) overlap including primitive norms and the 'N' factor."""
    geo = numpy.asarray(geo, dtype=numpy.float64)
    lxlylz = ao_spec.get_lxlylz()
    ncart = ao_spec.get_nlxlylz_per_cont()
    prim = ao_spec.get_prim_coeffs()
    npr = ao_spec.get_nprim_per_cont()
    atoms = ao_spec.get_assign_cont_to_atoms()
    isnorm = ao_spec.get_normalized()
    nshell = len(ncart)
    cart_off = numpy.concatenate([[0], numpy.cumsum(ncart)])
    nao = cart_off[-1]
    shell_of_prim = numpy.repeat(numpy.arange(nshell), npr)
    L_shell = numpy.array([lxlylz[cart_off[s]].sum() for s in range(nshell)])
    pL = L_shell[shell_of_prim]
    palpha = prim[:, 0]
    pcoef = prim[:, 1]
    pcent = geo[atoms[shell_of_prim]]
    S = numpy.zeros(nao * nao)
    for la in numpy.unique(pL):
        P = numpy.nonzero(pL == la)[0]
        for lb in numpy.unique(pL):
            Q = numpy.nonzero(pL == lb)[0]
            for p0 in range(0, len(P), 2048):
                pi = P[p0:p0 + 2048]
                ii, jj = numpy.meshgrid(pi, Q, indexing="ij")
                ii = ii.ravel()
                jj = jj.ravel()
                a = palpha[ii]
                b = palpha[jj]
                p = a + b
                mu = a * b / p
                AB = pcent[ii] - pcent[jj]
                r2 = (AB * AB).sum(1)
                keep = mu * r2 < _SCREEN
                if not keep.any():
                    continue
                ii, jj, a, b, p, mu, r2 = ii[keep], jj[keep], a[keep], b[keep], p[keep], mu[keep], r2[keep]
                A = pcent[ii]
                B = pcent[jj]
                Pc = (a[:, None] * A + b[:, None] * B) / p[:, None]
                pref = numpy.exp(-mu * r2) * (numpy.pi / p) ** 1.5 * pcoef[ii] * pcoef[jj]
                oo2p = 0.5 / p
                tabs = [_os_1d(Pc[:, d] - A[:, d], Pc[:, d] - B[:, d], oo2p, int(la), int(lb)) for d in range(3)]
                si = shell_of_prim[ii]
                sj = shell_of_prim[jj]
                # shells of one L may still list different component counts (custom lxlylz)
                ncomp_a = ncart[si]
                ncomp_b = ncart[sj]
                for ca in range(int(ncomp_a.max())):
                    ma = ca < ncomp_a
                    for cb in range(int(ncomp_b.max())):
                        m = ma & (cb < ncomp_b)
                        if not m.any():
                            continue
                        ra = cart_off[si[m]] + ca
                        rb = cart_off[sj[m]] + cb
                        la3 = lxlylz[ra]
                        lb3 = lxlylz[rb]
                        val = pref[m].copy()
                        for d in range(3):
                            tab = tabs[d]
                            fac = numpy.empty(m.sum())
                            for (x, y) in set(zip(la3[:, d].tolist(), lb3[:, d].tolist())):
                                sel = (la3[:, d] == x) & (lb3[:, d] == y)
                                fac[sel] = tab[x][y][m][sel]
                            val *= fac
                        na = numpy.ones(m.sum())
                        nb = numpy.ones(m.sum())
                        if not isnorm:
                            for (l, mm, n) in set(map(tuple, la3.tolist())):
                                sel = (la3 == (l, mm, n)).all(1)
                                na[sel] = ao_norm(l, mm, n, a[m][sel])
                            for (l, mm, n) in set(map(tuple, lb3.tolist())):
                                sel = (lb3 == (l, mm, n)).all(1)
                                nb[sel] = ao_norm(l, mm, n, b[m][sel])
                        S += numpy.bincount(ra * nao + rb, weights=val * na * nb, minlength=nao * nao)
    S = S.reshape(nao, nao)
    if "N" in ao_spec[0]:
        N = numpy.asarray(ao_spec[0]["N"], dtype=numpy.float64).reshape(-1)
        S *= N[:, None] * N[None, :]
    return S


def spherical_transform(ao_spec):
    """(NAOsph, NAOcart) matrix T with AO_sph = T @ AO_cart, evaluated the way
    orbkit's cartesian2spherical does it (core.py:135-176): for each listed
    component the *last* matching Cartesian row of the shell is used."""
    lxlylz = ao_spec.get_lxlylz()
    assign = ao_spec.get_assign_lxlylz_to_cont()
    sph = ao_spec.get_old_ao_spherical()
    rows = {}
    for i, j in enumerate(assign):
        rows.setdefault(int(j), []).append(i)
    T = numpy.zeros((len(sph), len(lxlylz)))
    for i0, (j0, k0) in enumerate(sph):
        comps, coefs, fac = get_cart2sph(*k0)
        for c, cf in zip(comps, coefs):
            idx = None
            for i in rows[int(j0)]:
                if tuple(lxlylz[i]) == tuple(c):
                    idx = i
            if idx is None:
                raise ValueError("spherical component %s not present in shell %d" % (c, j0))
            T[i0, idx] += cf * fac
    return T


def ao_overlap(geo, ao_spec):
    """Overlap in the output AO basis (spherical if ``ao_spec.spherical``)."""
    S = cartesian_overlap(geo, ao_spec)
    if getattr(ao_spec, "spherical", False):
        T = spherical_transform(ao_spec)
        S = T @ S @ T.T
    return S
