"""Basis set and one-electron multipole integrals for the CPU oracle (test infrastructure only).

Restates, in vectorised NumPy, the reference's
* ``newBasisset``            src/xtb/basisset.f90:33-308 (+ ``set_d_function`` :497-546)
* ``slaterToGauss``          src/slater.f90:373-483 (Stewart 1970 STO-nG, normalised)
* ``build_SDQH0``            src/xtb/hamiltonian.F90:146-371
* ``get_multiints`` / ``multipole_3d`` / ``olapp``   src/intgrad.f90:95-111,509-555,879-955
* ``get_grad_multiint`` / ``multipole_grad_3d`` / ``shiftintg``  src/intgrad.f90:607-728,958-1035
* ``dtrf2`` (Cartesian -> spherical d)  src/intgrad.f90:144-231
* ``h0scal`` / ``shellPoly``  src/scc_core.f90:644-680,728-754; ``dshellPoly`` src/grad_core.f90:40-72

Integrals are evaluated per primitive pair by expanding each Cartesian factor
about the Gaussian-product centre P (a horizontal shift), which is the same
published Obara-Saika-style route the reference takes; the screening rules
(primitive prefactor cut ``intcut`` and the 2000 bohr^2 pair cut) are kept
identical so that the same integrals are dropped.
"""
from math import comb

import numpy as np

from .params import AUTOEV, EVTOAU, PI, get_params

CART = {0: [(0, 0, 0)],
        1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
        2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]}
NCART = {0: 1, 1: 3, 2: 6}
NSPH = {0: 1, 1: 3, 2: 5}
# d-shell Cartesian -> spherical rows (dx2-y2, dz2, dxy, dxz, dyz), src/intgrad.f90:150-164
_S3 = np.sqrt(3.0)
DTRAFO = np.array([[0.5 * _S3, -0.5 * _S3, 0.0, 0.0, 0.0, 0.0],
                   [0.5, 0.5, -1.0, 0.0, 0.0, 0.0],
                   [0.0, 0.0, 0.0, 1.0, 0.0, 0.0],
                   [0.0, 0.0, 0.0, 0.0, 1.0, 0.0],
                   [0.0, 0.0, 0.0, 0.0, 0.0, 1.0]])
D_CART_SCALE = np.array([1.0, 1.0, 1.0, _S3, _S3, _S3])   # set_d_function trafo(5:10)
# moment components: 0 = S, 1..3 = x,y,z, 4..9 = xx,yy,zz,xy,xz,yz
MOMENTS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1),
           (2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
MAX_R2 = 2000.0
DFACT = [1.0, 1.0, 3.0, 15.0, 105.0, 945.0, 10395.0, 135135.0]


def slater_to_gauss(ng, n, l, zeta):
    """Stewart STO-nG expansion with normalisation, src/slater.f90:373-483."""
    P = get_params()
    ityp = {0: n, 1: 4 + n, 2: 7 + n, 3: 9 + n}[l] - 1
    if ng == 1:
        a = np.array([P.sto_alpha1[ityp]]) * zeta ** 2
        c = np.array([1.0])
    elif ng == 6 and n == 6:
        a = (P.sto_pAlpha6s if l == 0 else P.sto_pAlpha6p) * zeta ** 2
        c = (P.sto_pCoeff6s if l == 0 else P.sto_pCoeff6p).copy()
    else:
        a = getattr(P, f"sto_alpha{ng}")[:, ityp] * zeta ** 2
        c = getattr(P, f"sto_coeff{ng}")[:, ityp].copy()
    top = 2.0 / PI
    c = c * (top * a) ** 0.75 * np.sqrt(4 * a) ** l / np.sqrt(DFACT[l])
    return a, c


class Basis:
    """Shell/AO layout of a molecule (GFN2 valence basis; s, p and d shells)."""

    def __init__(self, Z):
        P = get_params()
        self.Z = np.asarray(Z, dtype=np.int64)
        sh_atom, sh_l, sh_zeta, sh_alpha, sh_coef, sh_nprim, sh_ao, sh_idx = [], [], [], [], [], [], [], []
        ao = 0
        for iat, z in enumerate(self.Z):
            iz = z - 1
            for ish in range(P.nShell[iz]):
                l = int(P.angShell[ish, iz])
                n = int(P.principalQuantumNumber[ish, iz])
                zeta = P.slaterExponent[ish, iz]
                ng = int(P.numberOfPrimitives[ish, iz])
                if not P.valenceShell[ish, iz]:
                    raise NotImplementedError("non-valence shells do not occur in GFN2")
                a, c = slater_to_gauss(ng, n, l, zeta)
                sh_atom.append(iat)
                sh_l.append(l)
                sh_zeta.append(zeta)
                sh_alpha.append(a)
                sh_coef.append(c)
                sh_nprim.append(ng)
                sh_ao.append(ao)
                sh_idx.append(ish)
                ao += NSPH[l]
        self.nshell = len(sh_atom)
        self.nao = ao
        self.sh_atom = np.array(sh_atom, dtype=np.int64)
        self.sh_l = np.array(sh_l, dtype=np.int64)
        self.sh_zeta = np.array(sh_zeta)
        self.sh_nprim = np.array(sh_nprim, dtype=np.int64)
        self.sh_ao = np.array(sh_ao, dtype=np.int64)
        self.sh_ish = np.array(sh_idx, dtype=np.int64)     # shell index within its element
        self.maxprim = max(sh_nprim) if sh_nprim else 1
        self.alpha = np.zeros((self.nshell, self.maxprim))
        self.coef = np.zeros((self.nshell, self.maxprim))
        for k in range(self.nshell):
            self.alpha[k, :sh_nprim[k]] = sh_alpha[k]
            self.coef[k, :sh_nprim[k]] = sh_coef[k]
        self.alpha[self.alpha == 0.0] = 1.0               # padded primitives carry zero coefficient
        self.ao_shell = np.repeat(np.arange(self.nshell), [NSPH[l] for l in sh_l])
        self.ao_atom = self.sh_atom[self.ao_shell]
        self.nat = len(self.Z)


def _olapp(m, gam):
    """Normalised 1D Gaussian moment <u^m>, src/intgrad.f90:95-111."""
    if m % 2:
        return np.zeros_like(gam)
    h = m // 2
    return (0.5 / gam) ** h * DFACT[h]


def _mom1d(i, j, PA, PB, PC, gam, orders):
    """1D integrals int (x-A)^i (x-B)^j (x-C)^e exp(-gam (x-P)^2) / sqrt(pi/gam) for e in orders."""
    out = {e: np.zeros_like(gam) for e in orders}
    if i < 0:
        return out
    t = [None] * (i + j + 3)
    for m in range(i + j + 3):
        t[m] = _olapp(m, gam)
    for a in range(i + 1):
        ca = comb(i, a) * PA ** (i - a)
        for b in range(j + 1):
            cab = ca * comb(j, b) * PB ** (j - b)
            m = a + b
            for e in orders:
                if e == 0:
                    v = t[m]
                elif e == 1:
                    v = t[m + 1] + PC * t[m]
                else:
                    v = t[m + 2] + 2 * PC * t[m + 1] + PC * PC * t[m]
                out[e] = out[e] + cab * v
    return out


def _sph(block, li, lj):
    """Cartesian -> spherical on the trailing two axes [.., cart_i, cart_j] (dtrf2)."""
    if li == 2:
        block = np.einsum("si,...ij->...sj", DTRAFO, block)
    if lj == 2:
        block = np.einsum("sj,...ij->...is", DTRAFO, block)
    return block


def pair_moments(basis, ish, jsh, RA, RB, RC, intcut, grad=False, grad_shift=False):
    """Moment integrals for a batch of shell pairs with equal (l_i, l_j).

    Returns array [npair, 10, nsph_i, nsph_j] of <i|M_k(C)|j> for the 10 moments
    (origin C per pair).  With ``grad`` returns additionally the derivative
    with respect to the centre A of shell i, [npair, 3, 10, nsph_i, nsph_j];
    with ``grad_shift`` that derivative includes the moment origin moving with
    A (``shiftintg`` moments 11-19) and C must equal A.
    """
    li = int(basis.sh_l[ish[0]])
    lj = int(basis.sh_l[jsh[0]])
    npair = len(ish)
    ai = basis.alpha[ish][:, :, None]        # [np, pi, 1]
    aj = basis.alpha[jsh][:, None, :]        # [np, 1, pj]
    ci = basis.coef[ish][:, :, None]
    cj = basis.coef[jsh][:, None, :]
    rab = RA - RB
    r2 = np.sum(rab * rab, axis=1)[:, None, None]
    gam = ai + aj
    est = r2 * ai * aj
    keep = (est <= intcut * gam) & (r2 <= MAX_R2) & (ci != 0) & (cj != 0)
    ab = 1.0 / gam
    kab = np.exp(-est * ab) * (np.sqrt(PI) * np.sqrt(ab)) ** 3
    cc = np.where(keep, kab * ci * cj, 0.0)
    Pc = (ai[..., None] * RA[:, None, None, :] + aj[..., None] * RB[:, None, None, :]) * ab[..., None]
    PA = Pc - RA[:, None, None, :]
    PB = Pc - RB[:, None, None, :]
    PC = Pc - RC[:, None, None, :]
    cart_i, cart_j = CART[li], CART[lj]
    nci, ncj = len(cart_i), len(cart_j)
    ints = np.zeros((npair, 10, nci, ncj))
    dints = np.zeros((npair, 3, 10, nci, ncj)) if grad else None
    # cache 1D integrals per axis, power pair
    cache = {}

    def one_d(ax, i, j):
        key = (ax, i, j)
        if key not in cache:
            cache[key] = _mom1d(i, j, PA[..., ax], PB[..., ax], PC[..., ax], gam, (0, 1, 2))
        return cache[key]

    for a, (ix, iy, iz) in enumerate(cart_i):
        pw_i = (ix, iy, iz)
        for b, (jx, jy, jz) in enumerate(cart_j):
            pw_j = (jx, jy, jz)
            vals = [one_d(ax, pw_i[ax], pw_j[ax]) for ax in range(3)]
            for k, (ex, ey, ez) in enumerate(MOMENTS):
                e = (ex, ey, ez)
                v = vals[0][e[0]] * vals[1][e[1]] * vals[2][e[2]]
                ints[:, k, a, b] = np.sum(cc * v, axis=(1, 2))
            if grad:
                for c in range(3):
                    up = one_d(c, pw_i[c] + 1, pw_j[c])
                    dn = one_d(c, pw_i[c] - 1, pw_j[c]) if pw_i[c] > 0 else None
                    for k, e in enumerate(MOMENTS):
                        fac = [vals[ax][e[ax]] for ax in range(3)]
                        g = 2 * ai * up[e[c]]
                        if dn is not None:
                            g = g - pw_i[c] * dn[e[c]]
                        fac[c] = g
                        dints[:, c, k, a, b] = np.sum(cc * fac[0] * fac[1] * fac[2], axis=(1, 2))
    # contraction coefficients of d Cartesian components
    if li == 2:
        ints = ints * D_CART_SCALE[None, None, :, None]
        if grad:
            dints = dints * D_CART_SCALE[None, None, None, :, None]
    if lj == 2:
        ints = ints * D_CART_SCALE[None, None, None, :]
        if grad:
            dints = dints * D_CART_SCALE[None, None, None, None, :]
    if grad and grad_shift:
        # moment origin moves with A: d/dA_c M_e = (...) - e_c * M_{e - 1_c}
        idx = {m: k for k, m in enumerate(MOMENTS)}
        for k, e in enumerate(MOMENTS):
            for c in range(3):
                if e[c] > 0:
                    lower = list(e)
                    lower[c] -= 1
                    dints[:, c, k] -= e[c] * ints[:, idx[tuple(lower)]]
    ints = _sph(ints, li, lj)
    if grad:
        dints = _sph(dints, li, lj)
    return ints, dints


def _pair_groups(basis, pairs_i, pairs_j):
    key = basis.sh_l[pairs_i] * 4 + basis.sh_l[pairs_j]
    for k in np.unique(key):
        sel = np.nonzero(key == k)[0]
        yield sel


def shell_pair_lists(basis):
    """All shell pairs on different atoms with atom(i) > atom(j)."""
    ns = basis.nshell
    ii, jj = np.meshgrid(np.arange(ns), np.arange(ns), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    m = basis.sh_atom[ii] > basis.sh_atom[jj]
    return ii[m], jj[m]


def h0_pair_factor(basis, cn_self, ish, jsh, xyz):
    """hav * shpoly of build_SDQH0 (eV) per shell pair (without the overlap)."""
    P = get_params()
    Zi = basis.Z[basis.sh_atom[ish]] - 1
    Zj = basis.Z[basis.sh_atom[jsh]] - 1
    li, lj = basis.sh_l[ish], basis.sh_l[jsh]
    hii, hjj = cn_self[ish], cn_self[jsh]
    zi, zj = basis.sh_zeta[ish], basis.sh_zeta[jsh]
    zetaij = (2 * np.sqrt(zi * zj) / (zi + zj)) ** 0.5
    den = (P.paulingEN[Zi] - P.paulingEN[Zj]) ** 2
    enpoly = 1.0 + P.enScale[lj, li] * den * (1.0 + 0.0 * den)
    km = P.kScale[lj, li] * enpoly
    hav = 0.5 * km * (hii + hjj) * zetaij
    ra, rb = xyz[basis.sh_atom[ish]], xyz[basis.sh_atom[jsh]]
    rab = np.sqrt(np.sum((ra - rb) ** 2, axis=1))
    rr = P.atomicRad[Zj] + P.atomicRad[Zi]
    r = rab / rr
    rf1 = 1.0 + 0.01 * P.shellPoly[basis.sh_ish[ish], Zi] * np.sqrt(r)
    rf2 = 1.0 + 0.01 * P.shellPoly[basis.sh_ish[jsh], Zj] * np.sqrt(r)
    return hav, rf1 * rf2


def build_sdqh0(basis, xyz, self_energy, intcut):
    """S, D(3), Q(6) (origin 0) and H0 (eV), H0_noovlp (eV), full square matrices."""
    nao = basis.nao
    S = np.zeros((nao, nao))
    D = np.zeros((3, nao, nao))
    Q = np.zeros((6, nao, nao))
    H0 = np.zeros((nao, nao))
    H0n = np.zeros((nao, nao))
    origin = np.zeros(3)
    pi_, pj_ = shell_pair_lists(basis)
    for sel in _pair_groups(basis, pi_, pj_):
        ish, jsh = pi_[sel], pj_[sel]
        RA, RB = xyz[basis.sh_atom[ish]], xyz[basis.sh_atom[jsh]]
        ints, _ = pair_moments(basis, ish, jsh, RA, RB, np.broadcast_to(origin, RA.shape), intcut)
        hav, shp = h0_pair_factor(basis, self_energy, ish, jsh, xyz)
        ni, nj = ints.shape[2], ints.shape[3]
        for a in range(ni):
            for b in range(nj):
                ia = basis.sh_ao[ish] + a
                jb = basis.sh_ao[jsh] + b
                s = ints[:, 0, a, b]
                S[ia, jb] = s
                S[jb, ia] = s
                D[:, ia, jb] = ints[:, 1:4, a, b].T
                D[:, jb, ia] = ints[:, 1:4, a, b].T
                Q[:, ia, jb] = ints[:, 4:10, a, b].T
                Q[:, jb, ia] = ints[:, 4:10, a, b].T
                H0[ia, jb] = H0[jb, ia] = hav * shp * s
                H0n[ia, jb] = H0n[jb, ia] = hav * shp
    # same-atom blocks: S = 1 on the diagonal, H0 = self energy, D/Q from the integrals
    for k in range(basis.nshell):
        l = basis.sh_l[k]
        for a in range(NSPH[l]):
            i = basis.sh_ao[k] + a
            S[i, i] = 1.0
            H0[i, i] = self_energy[k]
            H0n[i, i] = self_energy[k]
    ns = basis.nshell
    ii, jj = np.meshgrid(np.arange(ns), np.arange(ns), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    m = (basis.sh_atom[ii] == basis.sh_atom[jj]) & (ii >= jj)
    pi_, pj_ = ii[m], jj[m]
    for sel in _pair_groups(basis, pi_, pj_):
        ish, jsh = pi_[sel], pj_[sel]
        RA = xyz[basis.sh_atom[ish]]
        ints, _ = pair_moments(basis, ish, jsh, RA, RA, np.broadcast_to(origin, RA.shape), intcut)
        ni, nj = ints.shape[2], ints.shape[3]
        for a in range(ni):
            for b in range(nj):
                ia = basis.sh_ao[ish] + a
                jb = basis.sh_ao[jsh] + b
                D[:, ia, jb] = ints[:, 1:4, a, b].T
                D[:, jb, ia] = ints[:, 1:4, a, b].T
                Q[:, ia, jb] = ints[:, 4:10, a, b].T
                Q[:, jb, ia] = ints[:, 4:10, a, b].T
    return S, D, Q, H0, H0n


def grad_sdqh0(basis, xyz, self_energy, dse_dcn, intcut, P, Pew, ves, vs, vd, vq, H0n):
    """Gradient of the overlap-, dipole- and quadrupole-dependent energy terms.

    Restates build_dSDQH0_noreset, src/xtb/hamiltonian.F90:575-792.
    ``ves`` per shell (Eh), ``vs``/``vd``/``vq`` per atom (Eh, atom-centred
    moments), ``P`` density, ``Pew`` energy-weighted density (Eh),
    ``H0n`` the H0 matrix without overlap (eV).  Returns (gradient[nat,3], dhdcn[nat]).
    """
    Pr = get_params()
    nat = basis.nat
    g = np.zeros((nat, 3))
    dhdcn = np.zeros(nat)
    pi_, pj_ = shell_pair_lists(basis)
    ra_all = xyz[basis.sh_atom[pi_]]
    rb_all = xyz[basis.sh_atom[pj_]]
    keep = np.sum((ra_all - rb_all) ** 2, axis=1) <= 1600.0
    pi_, pj_ = pi_[keep], pj_[keep]
    for sel in _pair_groups(basis, pi_, pj_):
        ish, jsh = pi_[sel], pj_[sel]
        iat, jat = basis.sh_atom[ish], basis.sh_atom[jsh]
        RA, RB = xyz[iat], xyz[jat]
        # moments about B (k = 0..9) and about A (shifted, k = 1..9)
        ints_b, dints_b = pair_moments(basis, ish, jsh, RA, RB, RB, intcut, grad=True)
        ints_a, dints_a = pair_moments(basis, ish, jsh, RA, RB, RA, intcut, grad=True, grad_shift=True)
        Zi = basis.Z[iat] - 1
        Zj = basis.Z[jat] - 1
        rij = RA - RB
        rab2 = np.sum(rij * rij, axis=1)
        rab = np.sqrt(rab2)
        rr = Pr.atomicRad[Zi] + Pr.atomicRad[Zj]
        t14 = np.sqrt(rab / rr)
        k1 = Pr.shellPoly[basis.sh_ish[ish], Zi] * 0.01
        k2 = Pr.shellPoly[basis.sh_ish[jsh], Zj] * 0.01
        t15 = k1 * t14
        t23 = k2 * t14
        shpoly = (1.0 + t15) * (1.0 + k2 * t14)
        dshpoly = ((t15 * (1.0 + t23) + (1.0 + t15) * k2 * t14) * 0.5 / rab2)[:, None] * rij
        hav = 0.5 * (self_energy[ish] + self_energy[jsh])
        ni, nj = ints_b.shape[2], ints_b.shape[3]
        gx = np.zeros((len(ish), 3))
        dcn = np.zeros(len(ish))
        for a in range(ni):
            for b in range(nj):
                ia = basis.sh_ao[ish] + a
                jb = basis.sh_ao[jsh] + b
                Pij = P[jb, ia]
                Hij = H0n[jb, ia] * EVTOAU
                HP = Hij * Pij
                Sij = ints_b[:, 0, a, b]
                dS = dints_b[:, :, 0, a, b]
                term = 2 * HP - 2 * Pew[jb, ia] - Pij * (ves[ish] + ves[jsh]) + Pij * (vs[iat] + vs[jat])
                gx += (2 * HP * Sij / shpoly)[:, None] * dshpoly + dS * term[:, None]
                dtmp = np.einsum("pck,pk->pc", dints_a[:, :, 1:4, a, b], vd[iat]) + \
                    np.einsum("pck,pk->pc", dints_b[:, :, 1:4, a, b], vd[jat])
                qtmp = np.einsum("pck,pk->pc", dints_a[:, :, 4:10, a, b], vq[iat]) + \
                    np.einsum("pck,pk->pc", dints_b[:, :, 4:10, a, b], vq[jat])
                gx += Pij[:, None] * (dtmp + qtmp)
                dcn += HP / hav * Sij
        np.add.at(dhdcn, iat, dcn * dse_dcn[ish])
        np.add.at(dhdcn, jat, dcn * dse_dcn[jsh])
        np.add.at(g, iat, gx)
        np.add.at(g, jat, -gx)
    # diagonal: dE/dCN from the self energies
    diagP = np.diag(P)
    np.add.at(dhdcn, basis.ao_atom, diagP * dse_dcn[basis.ao_shell] * EVTOAU)
    return g, dhdcn
