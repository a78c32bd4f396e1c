"""GFN2-xTB self-consistent-charge single point: CPU oracle (test infrastructure only).

A NumPy/SciPy restatement of the reference path ``xtb_singlepoint`` ->
``TxTBCalculator%singlepoint`` -> ``scf`` (src/scf_module.F90:74-920) with the
same LAPACK sequence for the generalised eigenproblem (``dpotrf`` once, then
``dsygst`` + ``dsyevd`` + ``dtrsm`` per iteration; src/mctc/lapack/eigensolve.F90:218-246).
It is the checker for the CUDA engine and the timed CPU baseline; it is never
called by the product path.

Function-by-function sources are cited in each docstring.
"""
import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack as lp
from scipy.special import erf

from . import integrals as I
from .params import (AATOAU, AES_DMP3, AES_DMP5, AES_EXP, AES_RMAX, AES_SHIFT, AUTOEV, D4_A1, D4_A2,
                     D4_ALP, D4_GA, D4_GC, D4_S6, D4_S8, D4_S9, D4_S10, D4_WF, EVTOAU, GEXP, KB, PI,
                     REP_KEXP, REP_KEXP_LIGHT, REP_REXP, get_params, valence_charge)

SQRTPI = np.sqrt(PI)


# --------------------------------------------------------------------------------------
# coordination numbers
# --------------------------------------------------------------------------------------
def _pairs(n):
    i, j = np.tril_indices(n, -1)
    return i, j


def cn_lp(Z, xyz, kind, cutoff=40.0):
    """getCoordinationNumberLP, src/disp/coordinationnumber.F90:304-479 (molecular case).

    kind 'gfn': gfnCount (k=10), covalentRadD3; kind 'cov': erfCount (k=7.5) with
    the EN covalency factor k4*exp(-(|dEN|+k5)^2/k6).  Returns cn[N], dcndr[N(a), N(b), 3]
    with dcndr[a, b] = dCN_b / dR_a.
    """
    P = get_params()
    n = len(Z)
    i, j = _pairs(n)
    rij = xyz[i] - xyz[j]
    r2 = np.sum(rij ** 2, axis=1)
    m = (r2 <= cutoff ** 2) & (r2 >= 1e-12)
    i, j, rij, r2 = i[m], j[m], rij[m], r2[m]
    r1 = np.sqrt(r2)
    rc = P.covalentRadD3[Z[i] - 1] + P.covalentRadD3[Z[j] - 1]
    if kind == "gfn":
        k = 10.0

        def ec(kk, r, r0):
            return 1.0 / (1.0 + np.exp(-kk * (r0 / r - 1.0)))

        def dec(kk, r, r0):
            e = np.exp(-kk * (r0 / r - 1.0))
            return (-kk * r0 * e) / (r ** 2 * ((e + 1.0) ** 2))

        cf = ec(k, r1, rc) * ec(2 * k, r1, rc + 2)
        df = dec(k, r1, rc) * ec(2 * k, r1, rc + 2) + ec(k, r1, rc) * dec(2 * k, r1, rc + 2)
        den = 1.0
    elif kind == "cov":
        k = 7.5
        cf = 0.5 * (1.0 + erf(-k * (r1 - rc) / rc))
        df = -k / SQRTPI / rc * np.exp(-k ** 2 * (r1 - rc) ** 2 / rc ** 2)
        k4, k5, k6 = 4.10451, 19.08857, 2 * 11.28174 ** 2
        en = P.paulingEN
        den = k4 * np.exp(-(np.abs(en[Z[i] - 1] - en[Z[j] - 1]) + k5) ** 2 / k6)
    else:
        raise ValueError(kind)
    countf = den * cf
    countd = (den * df / r1)[:, None] * rij
    cn = np.zeros(n)
    np.add.at(cn, i, countf)
    np.add.at(cn, j, countf)
    dcndr = np.zeros((n, n, 3))
    np.add.at(dcndr, (i, i), countd)
    np.add.at(dcndr, (j, j), -countd)
    np.add.at(dcndr, (i, j), countd)
    np.add.at(dcndr, (j, i), -countd)
    return cn, dcndr


def cn_erf_eeq(Z, xyz):
    """ncoord_erf (EEQ guess), src/disp/ncoord.f90:469-506 (single-precision radii)."""
    P = get_params()
    n = len(Z)
    i, j = _pairs(n)
    r2 = np.sum((xyz[j] - xyz[i]) ** 2, axis=1)
    m = r2 <= 1600.0
    i, j, r2 = i[m], j[m], r2[m]
    r = np.sqrt(r2)
    rco = P.rcovD4[Z[j] - 1] + P.rcovD4[Z[i] - 1]
    tmp = 0.5 * (1.0 + erf(-7.5 * (r - rco) / rco))
    cn = np.zeros(n)
    np.add.at(cn, i, tmp)
    np.add.at(cn, j, tmp)
    return cn


def cn_d4(Z, xyz):
    """ncoord_d4, src/disp/ncoord.f90:575-615 (single-precision radii and EN)."""
    P = get_params()
    n = len(Z)
    i, j = _pairs(n)
    r2 = np.sum((xyz[j] - xyz[i]) ** 2, axis=1)
    m = r2 <= 1600.0
    i, j, r2 = i[m], j[m], r2[m]
    r = np.sqrt(r2)
    rco = P.rcovD4[Z[j] - 1] + P.rcovD4[Z[i] - 1]
    k4, k5, k6 = 4.10451, 19.08857, 2 * 11.28174 ** 2
    den = k4 * np.exp(-(np.abs(P.enD4[Z[i] - 1] - P.enD4[Z[j] - 1]) + k5) ** 2 / k6)
    tmp = den * 0.5 * (1.0 + erf(-7.5 * (r - rco) / rco))
    cn = np.zeros(n)
    np.add.at(cn, i, tmp)
    np.add.at(cn, j, tmp)
    return cn


# --------------------------------------------------------------------------------------
# EEQ guess and shell charges
# --------------------------------------------------------------------------------------
def eeq_guess(Z, xyz, charge=0.0):
    """eeq_chrgeq_core (0D), src/eeq_model.f90:60-80,678-880 with the 2019 model."""
    P = get_params()
    n = len(Z)
    cn = cn_erf_eeq(Z, xyz)
    en, gam, kap, alp = (P.eeq_en[Z - 1], P.eeq_gam[Z - 1], P.eeq_kappa[Z - 1], P.eeq_alpha[Z - 1])
    m = n + 1
    A = np.zeros((m, m))
    X = np.zeros(m)
    tmp = kap / (np.sqrt(cn) + 1e-14)
    X[:n] = -en + tmp * cn
    d = xyz[:, None, :] - xyz[None, :, :]
    r = np.sqrt(np.sum(d * d, axis=2))
    g = 1.0 / np.sqrt(alp[:, None] ** 2 + alp[None, :] ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        Am = erf(g * r) / r
    np.fill_diagonal(Am, gam + np.sqrt(2.0 / PI) / alp)
    A[:n, :n] = Am
    A[n, :m] = 1.0
    A[:m, n] = 1.0
    A[n, n] = 0.0
    X[n] = charge
    lu, piv, sol, info = lp.dsysv(A, X, lower=0)
    if info > 0:
        raise RuntimeError("EEQ: Coulomb matrix is singular")
    return sol[:n]


def ini_qshell(basis, z, q):
    """iniqshell, src/scc_core.f90:1475-1506."""
    P = get_params()
    qsh = np.zeros(basis.nshell)
    k = 0
    for iat, Zi in enumerate(basis.Z):
        ntot = -1.0e-6
        for ish in range(P.nShell[Zi - 1]):
            zs = P.referenceOcc[ish, Zi - 1]
            ntot += zs
            if ntot > z[iat]:
                zs = 0.0
            qsh[k] = zs / z[iat] * q[iat]
            k += 1
    return qsh


def set_zshell(basis, z):
    """setzshell, src/scc_core.f90:1509-1542."""
    P = get_params()
    zsh = np.zeros(basis.nshell)
    k = 0
    for iat, Zi in enumerate(basis.Z):
        ntot = -1.0e-6
        for ish in range(P.nShell[Zi - 1]):
            zsh[k] = P.referenceOcc[ish, Zi - 1]
            ntot += zsh[k]
            if ntot > z[iat]:
                zsh[k] = 0.0
            k += 1
    return zsh


# --------------------------------------------------------------------------------------
# isotropic electrostatics
# --------------------------------------------------------------------------------------
def coulomb_matrix(basis, xyz):
    """getCoulombMatrixCluster with arithmetic hardness average, src/coulomb/klopmanohno.F90:257-312."""
    P = get_params()
    eta = P.shellHardnessSh[basis.sh_ish, basis.Z[basis.sh_atom] - 1]
    at = basis.sh_atom
    d = xyz[at][:, None, :] - xyz[at][None, :, :]
    r = np.sqrt(np.sum(d * d, axis=2))
    gij = 0.5 * (eta[:, None] + eta[None, :])
    with np.errstate(divide="ignore"):
        J = 1.0 / (r ** GEXP + gij ** (-GEXP)) ** (1.0 / GEXP)
    same = at[:, None] == at[None, :]
    J = np.where(same, gij, J)
    return J


def coulomb_grad(basis, xyz, qsh):
    """getCoulombDerivsCluster contracted with qsh, src/coulomb/klopmanohno.F90:471-573."""
    P = get_params()
    eta = P.shellHardnessSh[basis.sh_ish, basis.Z[basis.sh_atom] - 1]
    at = basis.sh_atom
    d = xyz[at][None, :, :] - xyz[at][:, None, :]          # vec = R_j - R_i  [i, j]
    r = np.sqrt(np.sum(d * d, axis=2))
    gij = 0.5 * (eta[:, None] + eta[None, :])
    diff = at[:, None] > at[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        g1 = 1.0 / (r ** GEXP + gij ** (-GEXP))
        fac = -(r ** (GEXP - 2.0)) * g1 * g1 ** (1.0 / GEXP)
    fac = np.where(diff, fac, 0.0) * qsh[:, None] * qsh[None, :]
    dG = fac[:, :, None] * d                                  # [i, j, 3]
    g = np.zeros((basis.nat, 3))
    np.add.at(g, at, -np.sum(dG, axis=1))
    np.add.at(g, at, np.sum(dG, axis=0))
    return g


# --------------------------------------------------------------------------------------
# anisotropic electrostatics (AES)
# --------------------------------------------------------------------------------------
def _lin(i, j):
    a, b = max(i, j), min(i, j)
    return a * (a + 1) // 2 + b          # 0-based packed index of (i, j)


def aes_radii(Z, cn):
    """get_radcn, src/aespot.F90:1267-1281."""
    P = get_params()
    rco = P.multiRad[Z - 1]
    t1 = cn - P.valenceCN[Z - 1] - AES_SHIFT
    return rco + (AES_RMAX - rco) / (1.0 + np.exp(-AES_EXP * t1))


def aes_dradcn(Z, cn):
    """dradcn factor, src/aespot.F90:1292-1307."""
    P = get_params()
    rco = P.multiRad[Z - 1]
    t1 = np.exp(-AES_EXP * (cn - P.valenceCN[Z - 1] - AES_SHIFT))
    t2 = (AES_RMAX - rco) / (1.0 + 2.0 * t1 + t1 * t1)
    return t2 * AES_EXP * t1


def aes_gab(xyz, radcn):
    """mmomgabzero, src/aespot.F90:1219-1255 (+ dzero/gab :1309-1329)."""
    n = len(radcn)
    d = xyz[None, :, :] - xyz[:, None, :]
    r = np.sqrt(np.sum(d * d, axis=2))
    np.fill_diagonal(r, 1.0)
    rinv = 1.0 / r
    rco = 0.5 * (radcn[:, None] + radcn[None, :])
    damp3 = 1.0 / (1.0 + 6.0 * (rco * rinv) ** AES_DMP3)
    damp5 = 1.0 / (1.0 + 6.0 * (rco * rinv) ** AES_DMP5)
    gab3 = damp3 * rinv ** 3.0
    gab5 = damp5 * rinv ** 5.0
    np.fill_diagonal(gab3, 0.0)
    np.fill_diagonal(gab5, 0.0)
    return gab3, gab5


def mmompop(basis, xyz, P, S, D, Q):
    """Cumulative atomic dipole/quadrupole moments, mmompop_cpu src/aespot.F90:288-428.

    Returns dipm[N,3] and traceless qp[N,6] in packed order (xx, xy, yy, xz, yz, zz).
    """
    n = basis.nat
    at = basis.ao_atom
    ps = P * S
    pd = P[None] * D          # [3, nao, nao]
    pq = P[None] * Q          # [6, nao, nao]   (xx,yy,zz,xy,xz,yz)
    R = xyz[at]               # position of the atom of the ROW ao
    dip = np.zeros((n, 3))
    qp = np.zeros((n, 6))
    rs = ps.sum(axis=1)       # sum over nu of P S for each mu
    rd = pd.sum(axis=2)       # [3, nao]
    rq = pq.sum(axis=2)       # [6, nao]
    qidx = {(0, 0): 0, (1, 1): 1, (2, 2): 2, (1, 0): 3, (2, 0): 4, (2, 1): 5}
    for k in range(3):
        np.add.at(dip[:, k], at, R[:, k] * rs - rd[k])
    for k in range(3):
        for l in range(k + 1):
            kl = k * (k + 1) // 2 + l
            if k == l:
                t = 2.0 * rd[k] * R[:, k] - R[:, k] * R[:, k] * rs - rq[qidx[(k, k)]]
            else:
                t = rd[k] * R[:, l] + rd[l] * R[:, k] - R[:, l] * R[:, k] * rs - rq[qidx[(k, l)]]
            np.add.at(qp[:, kl], at, t)
    tr = 0.5 * (qp[:, 0] + qp[:, 2] + qp[:, 5])
    qp = 1.5 * qp
    qp[:, 0] -= tr
    qp[:, 2] -= tr
    qp[:, 5] -= tr
    return dip, qp


_IDX = np.array([[0, 1, 3], [1, 2, 4], [3, 4, 5]])   # packed index of (k, l)


def _full_q(qp):
    return qp[:, _IDX]                                   # [N, 3, 3]


def aniso_electro(Z, xyz, q, dipm, qp, gab3, gab5):
    """aniso_electro_cpu, src/aespot.F90:566-664.  Returns (e_aes, e_axc)."""
    P = get_params()
    Qf = _full_q(qp)
    tt = np.sum(dipm * dipm, axis=1)
    tt3 = np.sum(Qf * Qf, axis=(1, 2))
    epol = np.sum(P.dipKernel[Z - 1] * tt + tt3 * P.quadKernel[Z - 1])
    i, j = _pairs(len(Z))
    rij = xyz[j] - xyz[i]
    r2 = np.sum(rij * rij, axis=1)
    ed = q[j] * np.sum(dipm[i] * rij, axis=1) - q[i] * np.sum(dipm[j] * rij, axis=1)
    rr = rij[:, :, None] * rij[:, None, :]
    eq = q[j] * np.sum(Qf[i] * rr, axis=(1, 2)) + q[i] * np.sum(Qf[j] * rr, axis=(1, 2))
    edd = -3.0 * np.sum(dipm[j][:, :, None] * dipm[i][:, None, :] * rr, axis=(1, 2)) \
        + np.sum(dipm[j] * dipm[i], axis=1) * r2
    e = np.sum(ed * gab3[j, i]) + np.sum(eq * gab5[j, i]) + np.sum(edd * gab5[j, i])
    return e, epol


def setvsdq(Z, xyz, q, dipm, qp, gab3, gab5, shifted=True):
    """AES potentials vs[N], vd[N,3], vq[N,6] (qpint order xx,yy,zz,xy,xz,yz).

    shifted=True: setvsdq (origin-0 moment integrals, src/aespot.F90:727-848);
    shifted=False: setdvsdq (atom-centred moments, src/aespot.F90:861-952).
    """
    P = get_params()
    n = len(Z)
    Qf = _full_q(qp)
    ra = xyz[:, None, :]                 # i
    dra = xyz[:, None, :] - xyz[None, :, :]   # [i, j, 3] = R_i - R_j
    g3, g5 = gab3.T, gab5.T              # gab(j, i) as [i, j]
    qj = q[None, :]
    r2ab = np.sum(dra * dra, axis=2)
    t2a = np.sum(dipm[None, :, :] * dra, axis=2)
    qdd = np.einsum("jkl,ijk,ijl->ij", Qf, dra, dra)
    if shifted:
        r2a = np.sum(xyz * xyz, axis=1)[:, None]
        t1a = np.sum(ra * dra, axis=2)
        t3a = np.sum(ra * dipm[None, :, :], axis=2)
        rdr = ra * dra
        q4 = np.einsum("ijk,ijl->ij", rdr, rdr)
        dum5a = -qdd - 1.5 * qj * q4
        dum3a = -t1a * qj - t2a
        dum5a = dum5a + t3a * r2ab - 3.0 * t1a * t2a + 0.5 * qj * r2a * r2ab
    else:
        dum3a = -t2a
        dum5a = -qdd
    vs = np.sum(dum5a * g5 + dum3a * g3, axis=1)
    dd3 = dra * qj[..., None]
    dd5 = 3.0 * dra * t2a[..., None] - r2ab[..., None] * dipm[None, :, :]
    if shifted:
        dd5 = dd5 - (qj * r2ab)[..., None] * ra + 3.0 * (qj * t1a)[..., None] * dra
    vd = np.sum(dd3 * g3[..., None] + dd5 * g5[..., None], axis=1)
    # quadrupole potential in qpint order (xx, yy, zz, xy, xz, yz)
    vq = np.zeros((n, 6))
    w = (qj * g5)
    for l1 in range(3):
        vq[:, l1] = np.sum(-1.5 * w * dra[:, :, l1] * dra[:, :, l1] + 0.5 * r2ab * w, axis=1)
    for (l1, l2), ki in (((1, 0), 3), ((2, 0), 4), ((2, 1), 5)):
        vq[:, ki] = np.sum(-3.0 * w * dra[:, :, l2] * dra[:, :, l1], axis=1)
    # on-site kernel terms
    qs1 = P.dipKernel[Z - 1] * 2.0
    qs2 = P.quadKernel[Z - 1] * 6.0
    R = xyz
    if shifted:
        t3 = np.sum(R * dipm, axis=1) * qs1
    vd = vd - qs1[:, None] * dipm
    for l1 in range(3):
        for l2 in range(l1):
            ll = _lin(l1, l2)
            ki = l1 + l2 + 2
            vq[:, ki] -= qp[:, ll] * qs2
            if shifted:
                t3 -= R[:, l1] * R[:, l2] * qp[:, ll] * qs2
                vd[:, l1] += R[:, l2] * qp[:, ll] * qs2
                vd[:, l2] += R[:, l1] * qp[:, ll] * qs2
        ll = _lin(l1, l1)
        vq[:, l1] -= qp[:, ll] * qs2 * 0.5
        if shifted:
            t3 -= R[:, l1] * R[:, l1] * qp[:, ll] * qs2 * 0.5
            vd[:, l1] += R[:, l1] * qp[:, ll] * qs2
    tr = (qp[:, 0] + qp[:, 2] + qp[:, 5]) * P.quadKernel[Z - 1]
    if shifted:
        vs = vs + t3
    for l1 in range(3):
        vq[:, l1] += tr
        if shifted:
            vd[:, l1] -= 2.0 * R[:, l1] * tr
            vs = vs + tr * R[:, l1] * R[:, l1]
    return vs, vd, vq


def aniso_grad(Z, xyz, q, dipm, qp, radcn, dradcn_dr, gab3, gab5):
    """aniso_grad, src/aespot.F90:1060-1165.  dradcn_dr[a, i, 3] = dR0_i/dR_a."""
    n = len(Z)
    Qf = _full_q(qp)
    g = np.zeros((n, 3))
    rij = xyz[None, :, :] - xyz[:, None, :]           # [i, j] = R_j - R_i
    r2 = np.sum(rij * rij, axis=2)
    np.fill_diagonal(r2, 1.0)
    rabi = 1.0 / np.sqrt(r2)
    off = ~np.eye(n, dtype=bool)
    rco = 0.5 * (radcn[:, None] + radcn[None, :])

    def dz(dex):
        damp = 1.0 / (1.0 + 6.0 * (rco * rabi) ** dex)
        ddamp = -dex * rabi * (damp * damp - damp)
        return damp, ddamp

    damp1, dd1 = dz(AES_DMP3)
    damp2, dd2 = dz(AES_DMP5)
    dgab3 = (-3.0 * rabi * rabi ** 3.0) * damp1 + dd1 * rabi ** 3.0
    dgab5 = (-5.0 * rabi * rabi ** 5.0) * damp2 + dd2 * rabi ** 5.0
    G3, G5 = gab3.T, gab5.T                             # gab(j, i) as [i, j]
    qi, qj = q[:, None], q[None, :]
    di, dj = dipm[:, None, :], dipm[None, :, :]
    Qi, Qj = Qf[:, None], Qf[None, :]
    ed = qj * np.sum(di * rij, axis=2) - qi * np.sum(dj * rij, axis=2)
    rr = rij[..., :, None] * rij[..., None, :]
    eq = qj * np.sum(Qi * rr, axis=(2, 3)) + qi * np.sum(Qj * rr, axis=(2, 3))
    edd = -3.0 * np.einsum("ijk,ijl,ijkl->ij", np.broadcast_to(dj, rij.shape), np.broadcast_to(di, rij.shape), rr) \
        + np.sum(dj * di, axis=2) * r2
    ddm2 = np.sum(dj * di, axis=2)
    ddm3a = np.sum(di * rij, axis=2)
    ddm3b = np.sum(dj * rij, axis=2)
    qqa = np.einsum("ijl,jlk->ijk", rij, Qf)
    qqb = np.einsum("ijl,ilk->ijk", rij, Qf)
    tt = qi[..., None] * dj - qj[..., None] * di
    gk = G3[..., None] * tt
    gk += -2.0 * (G5 * ddm2)[..., None] * rij
    gk += 3.0 * (G5 * ddm3a)[..., None] * dj
    gk += 3.0 * (G5 * ddm3b)[..., None] * di
    gk += -2.0 * (G5 * qi)[..., None] * qqa
    gk += -2.0 * (G5 * qj)[..., None] * qqb
    dxi = rij * rabi[..., None]
    gk += -(ed * dgab3)[..., None] * dxi
    gk += -((eq + edd) * dgab5)[..., None] * dxi
    gk = np.where(off[..., None], gk, 0.0)
    g += np.sum(gk, axis=1)
    rab = 0.5 * (radcn[:, None] + radcn[None, :])
    tmp = ed * AES_DMP3 * G3 * (damp1 / rab) * (rab * rabi) ** AES_DMP3 + \
        (eq + edd) * AES_DMP5 * G5 * (damp2 / rab) * (rab * rabi) ** AES_DMP5
    tmp2 = 3.0 * np.sum(np.where(off, tmp, 0.0), axis=1)
    g -= np.einsum("i,aic->ac", tmp2, dradcn_dr)
    return g


# --------------------------------------------------------------------------------------
# D4 dispersion
# --------------------------------------------------------------------------------------
def _zeta(a, c, qref, qmod):
    qmod = np.asarray(qmod, dtype=float)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        v = np.exp(a * (1.0 - np.exp(c * (1.0 - qref / qmod))))
    return np.where(qmod < 0.0, np.exp(a), v)


def _dzeta(a, c, qref, qmod):
    qmod = np.asarray(qmod, dtype=float)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        v = -a * c * np.exp(c * (1.0 - qref / qmod)) * _zeta(a, c, qref, qmod) * qref / (qmod ** 2)
    return np.where(qmod < 0.0, 0.0, v)


_FREQ = np.array([0.000001, 0.05, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.2, 1.4, 1.6,
                  1.8, 2.0, 2.5, 3.0, 4.0, 5.0, 7.5, 10.0])
_W = np.zeros(23)
_W[0] = _FREQ[1] - _FREQ[0]
for _k in range(1, 22):
    _W[_k] = (_FREQ[_k] - _FREQ[_k - 1]) + (_FREQ[_k + 1] - _FREQ[_k])
_W[22] = _FREQ[22] - _FREQ[21]
_W *= 0.5


class D4Model:
    """newD4Model with p_refq_gfn2xtb reference charges, src/disp/dftd4.F90:106-203."""

    def __init__(self, elements):
        P = get_params()
        self.elements = sorted(set(int(e) for e in elements))
        self.nref, self.refcn, self.q, self.ncount, self.alpha = {}, {}, {}, {}, {}
        for ia in self.elements:
            a = ia - 1
            nref = int(P.d4_refn[a])
            cncount = np.zeros(19, dtype=int)
            cncount[0] = 1
            alph = np.zeros((nref, 23))
            for j in range(nref):
                is_ = int(P.d4_refsys[j, a])
                iz = P.d4_zeff[is_ - 1]
                sec_al = P.d4_sscale[is_ - 1] * P.d4_secaiw[:, is_ - 1] * \
                    _zeta(D4_GA, P.d4_gam[is_ - 1] * D4_GC, 0.0 + iz, P.d4_refh[j, a] + iz)
                icn = int(np.rint(P.d4_refcn[j, a]))
                cncount[icn] += 1
                alph[j] = np.maximum(P.d4_ascale[j, a] * (P.d4_alphaiw[:, j, a] - P.d4_hcount[j, a] * sec_al), 0.0)
            nc = np.zeros(nref, dtype=int)
            for j in range(nref):
                c = cncount[int(np.rint(P.d4_refcn[j, a]))]
                nc[j] = c * (c + 1) // 2
            self.nref[ia] = nref
            self.refcn[ia] = P.d4_refcovcn[:nref, a].copy()
            self.q[ia] = P.d4_refq[:nref, a].copy()
            self.ncount[ia] = nc
            self.alpha[ia] = alph
        self.c6 = {}
        thopi = 3.0 / PI
        for ia in self.elements:
            for ja in self.elements:
                self.c6[ia, ja] = thopi * (self.alpha[ia][:, None, :] * self.alpha[ja][None, :, :]) @ _W


def _gweights(model, Z, cn, with_deriv=False):
    """Gaussian CN weights of the reference systems (d4 :588-657 / weight_references :948-1065)."""
    out = []
    for iat, z in enumerate(Z):
        nref = model.nref[z]
        rcn = model.refcn[z]
        nc = model.ncount[z]
        expw = np.zeros(nref)
        expd = np.zeros(nref)
        for r in range(nref):
            for c in range(1, nc[r] + 1):
                twf = c * D4_WF
                val = -twf * (cn[iat] - rcn[r]) ** 2
                gw = 0.0 if val < -200.0 else np.exp(val)
                expw[r] += gw
                expd[r] += 2 * twf * (rcn[r] - cn[iat]) * gw
        norm = expw.sum()
        dnorm = expd.sum()
        norm = 1.0 / norm if norm > 1e-80 else 0.0
        gw = expw * norm
        dgw = expd * norm - expw * dnorm * norm ** 2
        if norm == 0.0:
            gw = np.where(np.abs(rcn.max() - rcn) < 1e-12, 1.0, 0.0)
        out.append((gw, dgw))
    return out


class SCD4:
    """Self-consistent D4 inside the SCC: TxTBDispersion, src/xtb/dispersion.f90:69-138."""

    def __init__(self, model, Z, xyz):
        P = get_params()
        self.model = model
        self.Z = Z
        cn = cn_d4(Z, xyz)
        self.off = np.concatenate([[0], np.cumsum([model.nref[z] for z in Z])])
        nd = self.off[-1]
        gw = np.zeros(nd)
        for iat, (g, _) in enumerate(_gweights(model, Z, cn)):
            gw[self.off[iat]:self.off[iat + 1]] = g
        self.gw = gw
        W = np.zeros((nd, nd))
        n = len(Z)
        sz = P.sqrtZr4r2
        for i in range(n):
            for j in range(i):
                ia, ja = Z[i], Z[j]
                r4r2 = 3.0 * sz[ia - 1] * sz[ja - 1]
                cut = D4_A1 * np.sqrt(r4r2) + D4_A2
                r2 = np.sum((xyz[j] - xyz[i]) ** 2)
                if r2 > 72.0 * 72.0:
                    continue
                oor6 = 1.0 / (r2 ** 3 + cut ** 6)
                oor8 = 1.0 / (r2 ** 4 + cut ** 8)
                oor10 = 1.0 / (r2 ** 5 + cut ** 10)
                gk = gw[self.off[i]:self.off[i + 1]]
                gl = gw[self.off[j]:self.off[j + 1]]
                gg = gk[:, None] * gl[None, :]
                c6 = model.c6[ia, ja]
                blk = gg * (-D4_S6 * c6 * oor6 - D4_S8 * (r4r2 * c6) * oor8 -
                            D4_S10 * (49.0 / 40.0 * r4r2 ** 2 * c6) * oor10)
                blk = np.where(gg < 1e-7, 0.0, blk)
                W[self.off[i]:self.off[i + 1], self.off[j]:self.off[j + 1]] = blk
                W[self.off[j]:self.off[j + 1], self.off[i]:self.off[i + 1]] = blk.T
        self.W = W

    def _zetavecs(self, q):
        P = get_params()
        nd = self.off[-1]
        zv = np.zeros(nd)
        dz = np.zeros(nd)
        for iat, z in enumerate(self.Z):
            sl = slice(self.off[iat], self.off[iat + 1])
            iz = P.d4_zeff[z - 1]
            gi = P.d4_gam[z - 1] * D4_GC
            m = self.gw[sl] >= 1e-7
            zz = _zeta(D4_GA, gi, self.model.q[z] + iz, q[iat] + iz)
            dd = _dzeta(D4_GA, gi, self.model.q[z] + iz, q[iat] + iz)
            zv[sl] = np.where(m, zz, 0.0)
            dz[sl] = np.where(m, dd, 0.0)
        return zv, dz

    def potential(self, q):
        """disppot, src/disp/dftd4.F90:735-818."""
        zv, dz = self._zetavecs(q)
        dum = self.W @ zv
        v = np.zeros(len(self.Z))
        np.add.at(v, np.repeat(np.arange(len(self.Z)), np.diff(self.off)), dum * dz)
        return v

    def energy(self, q):
        """edisp_scc, src/disp/dftd4.F90:821-864."""
        zv, _ = self._zetavecs(q)
        return float(zv @ (0.5 * (self.W @ zv)))


def d4_gradient(model, Z, xyz, q):
    """d4_full_gradient_latp for a molecule, src/disp/dftd4.F90:1624-1734 (+ :1832-2177, :2354-2433).

    Returns (e2body, e_atm, gradient[N,3]).
    """
    P = get_params()
    n = len(Z)
    cn, dcndr = cn_lp(Z, xyz, "cov", 40.0)
    zv, zr, zdcn, zrdcn = [], [], [], []
    for iat, (gw, dgw) in enumerate(_gweights(model, Z, cn, True)):
        z = Z[iat]
        zi = P.d4_zeff[z - 1]
        gi = D4_GC * P.d4_gam[z - 1]
        zq = _zeta(D4_GA, gi, model.q[z] + zi, q[iat] + zi)
        z0 = _zeta(D4_GA, gi, model.q[z] + zi, zi)
        zv.append(zq * gw)
        zr.append(z0 * gw)
        zdcn.append(zq * dgw)
        zrdcn.append(z0 * dgw)

    def atomic_c6(vec, dvec):
        c6 = np.zeros((n, n))
        dc6 = np.zeros((n, n))
        for i in range(n):
            for j in range(i + 1):
                rc6 = model.c6[Z[i], Z[j]]
                c6[i, j] = c6[j, i] = vec[i] @ rc6 @ vec[j]
                dc6[i, j] = dvec[i] @ rc6 @ vec[j]
                dc6[j, i] = vec[i] @ rc6 @ dvec[j]
        return c6, dc6

    c6, dc6 = atomic_c6(zv, zdcn)
    sz = P.sqrtZr4r2[Z - 1]
    g = np.zeros((n, 3))
    dEdcn = np.zeros(n)
    i, j = _pairs(n)
    rij = xyz[i] - xyz[j]
    r2 = np.sum(rij * rij, axis=1)
    m = (r2 <= 3600.0) & (r2 >= 1e-10)
    i, j, rij, r2 = i[m], j[m], rij[m], r2[m]
    r4r2 = 3 * sz[i] * sz[j]
    r0 = D4_A1 * np.sqrt(r4r2) + D4_A2
    t6 = 1.0 / (r2 ** 3 + r0 ** 6)
    t8 = 1.0 / (r2 ** 4 + r0 ** 8)
    t10 = 1.0 / (r2 ** 5 + r0 ** 10)
    d6 = -6 * r2 ** 2 * t6 ** 2
    d8 = -8 * r2 ** 3 * t8 ** 2
    d10 = -10 * r2 ** 4 * t10 ** 2
    disp = D4_S6 * t6 + D4_S8 * r4r2 * t8 + D4_S10 * 49.0 / 40.0 * r4r2 ** 2 * t10
    ddisp = D4_S6 * d6 + D4_S8 * r4r2 * d8 + D4_S10 * 49.0 / 40.0 * r4r2 ** 2 * d10
    e2 = np.sum(-c6[i, j] * disp)
    dG = (-c6[i, j] * ddisp)[:, None] * rij
    np.add.at(g, i, dG)
    np.add.at(g, j, -dG)
    np.add.at(dEdcn, i, -dc6[i, j] * disp)
    np.add.at(dEdcn, j, -dc6[j, i] * disp)
    # ATM three-body term with q = 0 reference charges
    c6z, dc6z = atomic_c6(zr, zrdcn)
    e3 = 0.0
    cut2 = 1600.0
    for ia in range(n):
        for ja in range(ia):
            rij_ = xyz[ja] - xyz[ia]
            r2ij = rij_ @ rij_
            if r2ij > cut2:
                continue
            ks = np.arange(ja)
            rik = xyz[ks] - xyz[ia]
            r2ik = np.sum(rik * rik, axis=1)
            rjk = xyz[ks] - xyz[ja]
            r2jk = np.sum(rjk * rjk, axis=1)
            mk = (r2ik <= cut2) & (r2jk <= cut2)
            ks, rik, r2ik, rjk, r2jk = ks[mk], rik[mk], r2ik[mk], rjk[mk], r2jk[mk]
            if len(ks) == 0:
                continue
            c6ij = c6z[ja, ia]
            c6ik = c6z[ks, ia]
            c6jk = c6z[ks, ja]
            cij = D4_A1 * np.sqrt(3.0 * sz[ia] * sz[ja]) + D4_A2
            cik = D4_A1 * np.sqrt(3.0 * sz[ia] * sz[ks]) + D4_A2
            cjk = D4_A1 * np.sqrt(3.0 * sz[ja] * sz[ks]) + D4_A2
            c9 = -np.sqrt(c6ij * c6ik * c6jk)
            ccc1 = cij * cjk * cik
            rrr2 = r2ij * r2jk * r2ik
            rrr1 = np.sqrt(rrr2)
            rrr3 = rrr1 * rrr2
            ang_fact = 0.375 / (rrr2 * rrr3)
            ang = ang_fact * (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik) * (-r2ij + r2jk + r2ik) + 1.0 / rrr3
            cralp = (ccc1 / rrr1) ** (float(D4_ALP) / 3.0)
            fdmp = 1.0 / (1.0 + 6.0 * cralp)
            dfdmp = -(2.0 * D4_ALP * cralp) * fdmp ** 2
            dE = -fdmp * ang * c9
            dang1 = -ang_fact * (r2ij ** 3 + r2ij ** 2 * (r2jk + r2ik) + r2ij * (3.0 * r2jk ** 2 + 2.0 * r2jk * r2ik + 3.0 * r2ik ** 2)
                                 - 5.0 * (r2jk - r2ik) ** 2 * (r2jk + r2ik))
            dGr1 = (-dang1 * c9 * fdmp + dfdmp * c9 * ang) / r2ij
            dang2 = -ang_fact * (r2ik ** 3 + r2ik ** 2 * (r2jk + r2ij) + r2ik * (3.0 * r2jk ** 2 + 2.0 * r2jk * r2ij + 3.0 * r2ij ** 2)
                                 - 5.0 * (r2jk - r2ij) ** 2 * (r2jk + r2ij))
            dGr2 = (-dang2 * c9 * fdmp + dfdmp * c9 * ang) / r2ik
            dang3 = -ang_fact * (r2jk ** 3 + r2jk ** 2 * (r2ik + r2ij) + r2jk * (3.0 * r2ik ** 2 + 2.0 * r2ik * r2ij + 3.0 * r2ij ** 2)
                                 - 5.0 * (r2ik - r2ij) ** 2 * (r2ik + r2ij))
            dGr3 = (-dang3 * c9 * fdmp + dfdmp * c9 * ang) / r2jk
            s = D4_S9
            e3 += np.sum(dE) * s
            g[ia] += s * (np.sum(-dGr1[:, None] * rij_[None, :], axis=0) + np.sum(-dGr2[:, None] * rik, axis=0))
            g[ja] += s * (np.sum(dGr1[:, None] * rij_[None, :], axis=0) + np.sum(-dGr3[:, None] * rjk, axis=0))
            np.add.at(g, ks, s * (dGr2[:, None] * rik + dGr3[:, None] * rjk))
            dc9 = 0.5 * c9 * (dc6z[ia, ja] / c6ij + dc6z[ia, ks] / c6ik)
            dEdcn[ia] += s * np.sum(-ang * fdmp * dc9)
            dc9 = 0.5 * c9 * (dc6z[ja, ia] / c6ij + dc6z[ja, ks] / c6jk)
            dEdcn[ja] += s * np.sum(-ang * fdmp * dc9)
            dc9 = 0.5 * c9 * (dc6z[ks, ia] / c6ik + dc6z[ks, ja] / c6jk)
            np.add.at(dEdcn, ks, s * (-ang * fdmp * dc9))
    g += np.einsum("abc,b->ac", dcndr, dEdcn)
    return e2, e3, g


# --------------------------------------------------------------------------------------
# repulsion
# --------------------------------------------------------------------------------------
def repulsion(Z, xyz, cutoff=40.0):
    """repulsionEnGrad_latp (molecular case), src/xtb/repulsion.F90:41-158."""
    P = get_params()
    n = len(Z)
    i, j = _pairs(n)
    rij = xyz[i] - xyz[j]
    r2 = np.sum(rij * rij, axis=1)
    m = (r2 <= cutoff ** 2) & (r2 >= 1e-8)
    i, j, rij, r2 = i[m], j[m], rij[m], r2[m]
    r1 = np.sqrt(r2)
    alpha = np.sqrt(P.repAlpha[Z[i] - 1] * P.repAlpha[Z[j] - 1])
    zeff = P.repZeff[Z[i] - 1] * P.repZeff[Z[j] - 1]
    kexp = np.where((Z[i] > 2) | (Z[j] > 2), REP_KEXP, REP_KEXP_LIGHT)
    t16 = r1 ** kexp
    t26 = np.exp(-alpha * t16)
    t27 = r1 ** REP_REXP
    dE = zeff * t26 / t27
    dG = (-(alpha * t16 * kexp + REP_REXP) * dE / r2)[:, None] * rij
    g = np.zeros((n, 3))
    np.add.at(g, i, dG)
    np.add.at(g, j, -dG)
    return float(np.sum(dE)), g


# --------------------------------------------------------------------------------------
# SCC helpers
# --------------------------------------------------------------------------------------
def occu(nao, nel, nopen):
    """occu, src/scc_core.f90:1112-1170: alpha/beta integer occupations."""
    focc = np.zeros(nao, dtype=int)
    if nel % 2 == 0:
        ihomo = nel // 2
        focc[:ihomo] = 2
        if 2 * ihomo != nel:
            ihomo += 1
            focc[ihomo - 1] = 1
            if nopen == 0:
                nopen = 1
        if nopen > 1:
            for i in range(1, nopen // 2 + 1):
                focc[ihomo - i] -= 1
                focc[ihomo + i - 1] += 1
    else:
        na = nel // 2 + (nopen - 1) // 2 + 1
        nb = nel // 2 - (nopen - 1) // 2
        focc[:na] += 1
        focc[:nb] += 1
    focca = np.where(focc >= 1, 1.0, 0.0)
    foccb = np.where(focc == 2, 1.0, 0.0)
    ihomoa = int(np.max(np.nonzero(focca > 0.99)[0]) + 1) if np.any(focca > 0.99) else 0
    ihomob = int(np.max(np.nonzero(foccb > 0.99)[0]) + 1) if np.any(foccb > 0.99) else 0
    return focca, foccb, ihomoa, ihomob


def fermismear(eig, nel, etemp):
    """fermismear, src/scc_core.f90:983-1064.  Returns (occ, e_fermi, -TS)."""
    norbs = len(eig)
    bkt = KB * AUTOEV * etemp
    thr = 1e-9
    occ = np.zeros(norbs)
    if nel + 1 > norbs:
        # no LUMO: the integer occupations from occu stay (src/scc_core.f90:1001-1004)
        ef = eig[nel - 1]
        occ[:nel] = 1.0
    elif nel == 0:
        ef = eig[0]
    else:
        ef = 0.5 * (eig[nel - 1] + eig[nel])
        occt = float(nel)
        for _ in range(200):
            x = (eig - ef) / bkt
            mask = x < 50
            ex = np.exp(np.where(mask, x, 0.0))
            f = np.where(mask, 1.0 / (ex + 1.0), 0.0)
            df = np.where(mask, ex / (bkt * (ex + 1.0) ** 2), 0.0)
            occ = f
            tot = np.sum(f)
            totd = np.sum(df)
            ef = ef + (occt - tot) / totd
            if abs(occt - tot) <= thr:
                break
    m = (occ > thr) & (1.0 - occ > thr)
    o = occ[m]
    s = np.sum(o * np.log(o) + (1.0 - o) * np.log(1.0 - o)) * KB * etemp
    return occ, ef, s


def broyden(q, qlast, dq, dqlast, it, alpha, st):
    """Modified Broyden mixing (Johnson 1988), src/broyden.f90:37-153.  ``st`` holds history."""
    omega0, minw, maxw, wfac = 0.01, 1.0, 100000.0, 0.01
    if it == 1:
        dqlast[:] = dq
        qlast[:] = q
        return q + alpha * dq
    it1 = it - 1
    om = np.sqrt(dq @ dq)
    om = wfac / om if om > wfac / maxw else maxw
    om = max(om, minw)
    st["omega"].append(om)
    df = dq - dqlast
    inv = 1.0 / np.sqrt(df @ df)
    df = inv * df
    st["df"].append(df)
    dfm = np.array(st["df"])
    a = dfm @ dfm.T
    omega = np.array(st["omega"])
    c = omega * (dfm @ dq)
    beta = omega[:, None] * omega[None, :] * a
    beta[np.diag_indices(it1)] += omega0 * omega0
    beta = np.linalg.inv(beta)
    gamma = c @ beta
    st["u"].append(alpha * df + inv * (q - qlast))
    dqlast[:] = dq
    qlast[:] = q
    qn = q + alpha * dq
    u = np.array(st["u"])
    qn = qn - (omega * gamma) @ u
    return qn


def setdq_masks(D, Q, neglect):
    """setdqlist screening, src/aespot.F90:34-85: boolean masks of significant D/Q pairs."""
    thr2 = neglect * 1.0e-2
    t1 = np.sum(D * D, axis=0)
    t2 = np.sum(Q[:3] * Q[:3], axis=0) + 2.0 * np.sum(Q[3:] * Q[3:], axis=0)
    return t1 > thr2, t2 > thr2


# --------------------------------------------------------------------------------------
# single point driver
# --------------------------------------------------------------------------------------
class Result:
    pass


def pc_potential(basis, xyz, pc_q, pc_xyz, pc_gam):
    """Shell potential of external point charges, jpot_pcem_gfn2 (src/embedding.f90:225-256):
    V_sh = sum_k q_k / sqrt(r^2 + 1/x^2), x = (eta_sh + gam_k) / 2."""
    P = get_params()
    eta = P.shellHardnessSh[basis.sh_ish, basis.Z[basis.sh_atom] - 1]
    d = xyz[basis.sh_atom][:, None, :] - pc_xyz[None, :, :]
    r2 = np.sum(d * d, axis=2)
    x = 0.5 * (eta[:, None] + pc_gam[None, :])
    return np.sum(pc_q[None, :] / np.sqrt(r2 + 1.0 / x ** 2), axis=1)


def pc_gradient(basis, xyz, qsh, pc_q, pc_xyz, pc_gam):
    """pcem_grad_gfn2 (src/embedding.f90:329-365): gradient on the atoms and on the charges."""
    P = get_params()
    eta = P.shellHardnessSh[basis.sh_ish, basis.Z[basis.sh_atom] - 1]
    dr = xyz[basis.sh_atom][:, None, :] - pc_xyz[None, :, :]          # [shell, pc, 3]
    r2 = np.sum(dr * dr, axis=2)
    rr = 1.0 / (0.5 * (eta[:, None] + pc_gam[None, :])) ** 2
    yy = qsh[:, None] * pc_q[None, :] * (r2 + rr) ** -1.5
    g = np.zeros((basis.nat, 3))
    np.add.at(g, basis.sh_atom, -np.sum(dr * yy[..., None], axis=1))
    gpc = np.sum(dr * yy[..., None], axis=0)
    return g, gpc


def singlepoint(Z, xyz, charge=0.0, uhf=0, etemp=300.0, accuracy=1.0, maxiter=250,
                guess="eeq", q_init=None, qsh_init=None, dipm_init=None, qp_init=None, verbose=False,
                pc_charges=None, pc_positions=None, pc_gam=None, solvation=None):
    """GFN2-xTB energy, charges and gradient for a molecule (Bohr in, Eh and Eh/bohr out).

    Follows scf, src/scf_module.F90:74-920, and scc, src/scc_core.f90:255-640.  External point
    charges (pc_charges[k], pc_positions[k, 3] in Bohr, pc_gam[k] hardness) add the shell
    potential of jpot_pcem_gfn2 to every iteration's shift (src/scc_core.f90:438), their energy
    (electro_pcem, src/embedding.f90:261-280) and gradient (src/embedding.f90:329-365).
    An implicit solvent (`solvation`, an oracle.solvation.Solvation of this molecule) is updated
    for the geometry once (src/scf_module.F90:298-321), adds B q to the atomic potential of every
    iteration (src/scc_core.f90:444-448) and its energy to the electronic energy
    (src/scc_core.f90:544-548), and its gradient after convergence (src/scf_module.F90:761-776).
    """
    Z = np.asarray(Z, dtype=np.int64)
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(Z)
    Pr = get_params()
    basis = I.Basis(Z)
    nao, nsh = basis.nao, basis.nshell
    zval = valence_charge(Z)
    # thresholds, src/scf_module.F90:266-277
    intcut = max(20.0, 25.0 - 10.0 * np.log10(accuracy))
    neglect = 10.0e-9 * accuracy
    scfconv = 1.0e-6 * accuracy
    qconv = 1.0e-4 * accuracy
    # initial guess (newWavefunction, src/xtb/calculator.f90:432-496)
    if q_init is not None:
        q = np.array(q_init, dtype=float)
    elif guess == "eeq":
        q = eeq_guess(Z, xyz, charge)
    else:
        q = np.full(n, charge / n)
    qsh = ini_qshell(basis, zval, q) if qsh_init is None else np.array(qsh_init, dtype=float)
    q = np.zeros(n)
    np.add.at(q, basis.sh_atom, qsh)
    dipm = np.zeros((n, 3)) if dipm_init is None else np.array(dipm_init, dtype=float)
    qp = np.zeros((n, 6)) if qp_init is None else np.array(qp_init, dtype=float)

    nel = int(round(np.sum(zval) - charge))
    nopen = uhf
    if nopen == 0 and nel % 2 != 0:
        nopen = 1
    zsh = set_zshell(basis, zval)
    focca, foccb, ihomoa, ihomob = occu(nao, nel, nopen)

    # classical terms
    erep, grad = repulsion(Z, xyz)
    cn, dcndr = cn_lp(Z, xyz, "gfn", 40.0)
    d4m = D4Model(Z)
    scd4 = SCD4(d4m, Z, xyz)
    # integrals
    se = Pr.selfEnergy[basis.sh_ish, Z[basis.sh_atom] - 1] - Pr.kCN[basis.sh_ish, Z[basis.sh_atom] - 1] * cn[basis.sh_atom]
    dse = -Pr.kCN[basis.sh_ish, Z[basis.sh_atom] - 1]
    S, D, Q, H0, H0n = I.build_sdqh0(basis, xyz, se, intcut)
    dmask, qmask = setdq_masks(D, Q, neglect)
    Dm = np.where(dmask[None], D, 0.0)
    Qm = np.where(qmask[None], Q, 0.0)
    radcn = aes_radii(Z, cn)
    gab3, gab5 = aes_gab(xyz, radcn)
    J = coulomb_matrix(basis, xyz)
    gam3 = Pr.thirdOrderShell[basis.sh_ish, Z[basis.sh_atom] - 1]
    pcem = pc_charges is not None and len(pc_charges) > 0
    if pcem:
        pc_q = np.asarray(pc_charges, dtype=float)
        pc_x = np.asarray(pc_positions, dtype=float).reshape(-1, 3)
        pc_g = np.asarray(pc_gam, dtype=float)
        vpc = pc_potential(basis, xyz, pc_q, pc_x, pc_g)
    else:
        vpc = np.zeros(nsh)

    if solvation is not None:
        solvation.update(xyz)

    # SCC, src/scc_core.f90:406-640
    U = sla.cholesky(S, lower=False)
    nbr = nsh + 9 * n
    st = {"omega": [], "df": [], "u": []}
    qlast = np.zeros(nbr)
    dqlast = np.zeros(nbr)
    eel = 0.0
    lastdiag = False
    converged = False
    ao_sh = basis.ao_shell
    ao_at = basis.ao_atom
    iters = 0
    for it in range(1, maxiter + 1):
        iters = it
        shift = vpc + J @ qsh + gam3 * qsh ** 2
        vs, vd, vq = setvsdq(Z, xyz, q, dipm, qp, gab3, gab5, shifted=True)
        atshift = scd4.potential(q)
        if solvation is not None:
            atshift = atshift + solvation.shift(q)
        shift = shift + atshift[basis.sh_atom]
        # buildIsoAnisotropicH1, src/scc_core.f90:154-251 (eV)
        dum = S * AUTOEV * 0.5
        H = H0 - dum * (shift[ao_sh][:, None] + shift[ao_sh][None, :]) \
            + dum * (vs[ao_at][:, None] + vs[ao_at][None, :])
        vdsum = vd[ao_at][:, None, :] + vd[ao_at][None, :, :]           # [nao, nao, 3]
        H += 0.5 * AUTOEV * np.einsum("kij,ijk->ij", Dm, vdsum)
        vqsum = vq[ao_at][:, None, :] + vq[ao_at][None, :, :]
        H += 0.5 * AUTOEV * np.einsum("kij,ijk->ij", Qm, vqsum)
        # generalised eigenproblem: dsygst + dsyevd + dtrsm
        A, info = lp.dsygst(H, U, itype=1, lower=0)
        if info != 0:
            raise RuntimeError("dsygst failed")
        emo, Zv, info = lp.dsyevd(A, compute_v=1, lower=0)
        if info != 0:
            raise RuntimeError("Diagonalization of Hamiltonian failed")
        C = sla.solve_triangular(U, Zv, lower=False)
        # Fermi smearing
        fa, efa, ga = fermismear(emo, ihomoa, etemp)
        fb, efb, gb = fermismear(emo, ihomob, etemp)
        focc = fa + fb
        q_in = np.concatenate([qsh, dipm.ravel(), qp.ravel()])
        Pm = (C * focc[None, :]) @ C.T
        # Mulliken shell populations
        ps = Pm * S
        pop = np.zeros(nsh)
        np.add.at(pop, ao_sh, ps.sum(axis=1))
        qsh = zsh - pop
        q = np.zeros(n)
        np.add.at(q, basis.sh_atom, qsh)
        eold = eel
        es = 0.5 * qsh @ (J @ qsh) + np.sum(gam3 * qsh ** 3 / 3.0)
        h = np.sum(np.tril(Pm, -1) * np.tril(H0, -1)) + 0.5 * np.sum(np.diag(Pm) * np.diag(H0))
        eel = es + 2.0 * h * EVTOAU
        ees = es
        dipm, qp = mmompop(basis, xyz, Pm, S, D, Q)
        eaes, epol = aniso_electro(Z, xyz, q, dipm, qp, gab3, gab5)
        eel += eaes + epol
        ed = scd4.energy(q)
        eel += ed
        epcem = float(qsh @ vpc)
        eel += epcem
        if solvation is not None:
            eel += solvation.energy(q)
        eel += ga + gb
        econv = abs(eel - eold) < scfconv
        dq = np.concatenate([qsh, dipm.ravel(), qp.ravel()]) - q_in
        rmsq = np.sqrt(np.sum(dq ** 2) / n)
        qconvd = rmsq < qconv
        if n > 1:
            qn = broyden(q_in.copy(), qlast, dq, dqlast, it, 0.4, st)
        else:
            qn = q_in + dq     # simple damping branch is never taken for GFN2 molecules > 1 atom
        qsh = qn[:nsh]
        dipm = qn[nsh:nsh + 3 * n].reshape(n, 3)
        qp = qn[nsh + 3 * n:].reshape(n, 6)
        q = np.zeros(n)
        np.add.at(q, basis.sh_atom, qsh)
        if verbose:
            print(f"{it:4d} {eel:15.7f} {eel - eold:14.6e} {rmsq:11.3e}")
        if econv and qconvd:
            converged = True
            if lastdiag:
                break
            lastdiag = True
    # gradient block, src/scf_module.F90:665-798
    Pew = (C * (focc * emo * EVTOAU)[None, :]) @ C.T
    vs2, vd2, vq2 = setvsdq(Z, xyz, q, dipm, qp, gab3, gab5, shifted=False)
    gh, dhdcn = I.grad_sdqh0(basis, xyz, se, dse, intcut, Pm, Pew, shift, vs2, vd2, vq2, H0n)
    grad += gh
    grad += np.einsum("abc,b->ac", dcndr, dhdcn)
    dr = aes_dradcn(Z, cn)
    grad += aniso_grad(Z, xyz, q, dipm, qp, radcn, dcndr * dr[None, :, None], gab3, gab5)
    e2, embd, gd4 = d4_gradient(d4m, Z, xyz, q)
    grad += gd4
    grad += coulomb_grad(basis, xyz, qsh)
    pcgrad = None
    if pcem:
        gpc_atoms, pcgrad = pc_gradient(basis, xyz, qsh, pc_q, pc_x, pc_g)
        grad += gpc_atoms
    esolv = None
    if solvation is not None:
        grad += solvation.gradient(q)
        esolv = sum(solvation.energy_parts(q))

    # dipole moment (calc_dipole, src/dipole.f90:94-128) and Wiberg-Mayer bond orders
    # (get_wiberg, src/scc_core.f90:1208-1245) from the last density
    dip = np.sum(xyz * zval[:, None], axis=0) - np.einsum("kij,ij->k", D, Pm)
    if ihomoa == ihomob:
        PSs, fac = [Pm @ S], 1.0
    else:   # get_unrestricted_wiberg, src/scc_core.f90:1248-1295
        PSs, fac = [((C * fa[None, :]) @ C.T) @ S, ((C * fb[None, :]) @ C.T) @ S], 2.0
    wbo = np.zeros((n, n))
    ao0 = basis.sh_ao[np.searchsorted(basis.sh_atom, np.arange(n))]
    ao1 = np.append(ao0[1:], nao)
    for i in range(n):
        for j in range(i):
            if np.sum((xyz[i] - xyz[j]) ** 2) < 100.0:
                tot = 0.0
                for PS in PSs:
                    tot += np.sum(PS[ao0[i]:ao1[i], ao0[j]:ao1[j]] * PS[ao0[j]:ao1[j], ao0[i]:ao1[i]].T)
                wbo[i, j] = wbo[j, i] = fac * tot

    r = Result()
    r.dipole = dip
    r.wbo = wbo
    r.energy = eel + erep + embd
    r.e_elec = eel + embd
    r.e_rep = erep
    r.e_es = ees
    r.e_aes = eaes
    r.e_axc = epol
    r.e_disp = ed + embd
    r.gradient = grad
    r.pcgrad = pcgrad
    r.e_solv = esolv
    r.gnorm = np.sqrt(np.sum(grad ** 2))
    r.q = q
    r.qsh = qsh
    r.dipm = dipm
    r.qp = qp
    r.emo = emo
    r.focc = focc
    r.P = Pm
    r.S = S
    r.D = D
    r.ihomo = ihomoa
    r.hl_gap = emo[ihomoa] - emo[ihomoa - 1] if 0 < ihomoa < nao else 0.0
    r.iterations = iters
    r.converged = converged
    r.nao = nao
    r.nshell = nsh
    r.basis = basis
    return r


def hessian(Z, xyz, charge=0.0, uhf=0, step=0.005, atoms=None, **kw):
    """Numerical Hessian (Eh/bohr^2) and dipole gradient by central differences of analytic
    gradients, as xtb_hessian does for a fresh results object (hessian_api,
    src/api/interface.f90:309-454; TCalculator%hessian, src/type/calculator.f90:116-199):
    every displaced single point starts from the initial-guess wavefunction of the
    undisplaced molecule (EEQ charges, iniqshell, zero multipoles), H[jj, ii] =
    (g_jj(+h) - g_jj(-h)) / 2h for displaced coordinate ii, then H is symmetrised.
    Returns (H [3N, 3N], dipgrad [3N, 3])."""
    Z = np.asarray(Z, dtype=np.int64)
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(Z)
    basis = I.Basis(Z)
    q0 = eeq_guess(Z, xyz, charge)
    qsh0 = ini_qshell(basis, valence_charge(Z), q0)
    atoms = range(n) if atoms is None else atoms
    H = np.zeros((3 * n, 3 * n))
    dipgrad = np.zeros((3 * n, 3))
    s2 = 0.5 / step
    for iat in atoms:
        for ic in range(3):
            ii = 3 * iat + ic
            res = []
            for sgn in (1.0, -1.0):
                x = xyz.copy()
                x[iat, ic] += sgn * step
                res.append(singlepoint(Z, x, charge=charge, uhf=uhf, qsh_init=qsh0, **kw))
            H[:, ii] += (res[0].gradient - res[1].gradient).ravel() * s2
            dipgrad[ii] = (res[0].dipole - res[1].dipole) * s2
    H = 0.5 * (H + H.T)
    return H, dipgrad
