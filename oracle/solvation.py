"""GBSA / ALPB implicit solvation for the CPU oracle (test infrastructure only).

A restatement, in vectorised NumPy, of the reference's generalised-Born model with a
solvent-accessible-surface term (GFN2 uses plain Mulliken charges, no CM5 correction):

* model set-up         src/solv/model.f90:510-545 (paramToModel), :150-161 (constants),
                       src/solv/state.f90 (solution-state shift), src/solv/gbsa.f90:217-389
                       (initBorn: kernel, keps, ALPB alpha/eps, radii, SASA switching, H-bond)
* Born radii (GBOBC-II) src/solv/born.f90 (compute_psi, compute_bornr)
* numerical SASA       src/solv/sasa.f90 (compute_numsa, compute_w_sp) on the Lebedev-Laikov
                       grid of src/solv/lebedev.f90
* Born matrix          src/solv/kernel.f90:586-760 (Still, P16 and the salt-screened Still
                       kernel), src/solv/gbsa.f90:445-491 (H-bond diagonal, ALPB shape term)
* shift and energy     src/solv/gbsa.f90:495-596 (addShift, getEnergy, getEnergyParts)
* gradient             src/solv/kernel.f90:171-378 (+ salt variant), src/solv/gbsa.f90:600-777
                       (SASA, H-bond and ALPB shape-term derivatives)

Inside the SCC the atomic potential gains B q (src/scc_core.f90:444-448) and the electronic
energy 1/2 q^T B q + G_sasa + G_shift (src/scc_core.f90:544-548); the gradient is added once
after convergence (src/scf_module.F90:761-776).

Tables (parameter sets, D3 van der Waals radii, Lebedev generators) come from
``xtb_gb300/data/solvation_params.json``, extracted by ``oracle/gen_solvation.py``.
"""
import itertools
import json
import os

import numpy as np

from .params import AATOAU, KB, PI

_JSON = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "xtb_gb300", "data",
                     "solvation_params.json")
_DATA = None

KCALTOAU = 1.0 / 627.50947428                 # src/mctc/convert.f90:31-32
MOLCM3TOAU = 8.92388e-2                       # src/solv/model.f90:153
SURFACE_TENSION = 1.0e-5                      # src/solv/model.f90:156
LRCUT = 35.0 * AATOAU                         # src/solv/model.f90:161 (Born radii pair cutoff)
ROFFSET = 2.0 * AATOAU                        # src/solv/model.f90:162 (SASA neighbour margin)
W = 0.3 * AATOAU                              # SASA switching half-width, src/solv/sasa.f90
AH0, AH1, AH3 = 0.5, 3.0 / (4.0 * W), -1.0 / (4.0 * W ** 3)
TOLSESP = 1.0e-6
OBC_ALPHA, OBC_BETA, OBC_GAMMA = 1.0, 0.8, 4.85   # src/solv/born.f90
ZETA_P16 = 1.028                              # src/solv/kernel.f90
ALPB_ALPHA = 0.571412                         # src/solv/gbsa.f90:245
KAPPA_CONST = 0.7897e-3                       # src/solv/gbsa.f90:88
TINY = np.finfo(float).tiny
# solution states, src/solv/state.f90
STATE_GSOLV, STATE_REFERENCE, STATE_MOL1BAR = 1, 2, 3

# solvent name aliases (src/solv/model.f90:215-249, normalizeSolventName) and the internal
# names of the GBSA sets that differ from the normalised ones (loadInternalParam, :280-300)
_ALIASES = {"methylcyanide": "acetonitrile", "methylenechloride": "ch2cl2", "dichloromethane": "ch2cl2",
            "dcm": "ch2cl2", "chloroform": "chcl3", "trichloromethane": "chcl3", "tcm": "chcl3",
            "carbondisulfide": "cs2", "diethylether": "ether", "dimethylformamide": "dmf",
            "dimethylsulfoxide": "dmso", "furan": "furane", "nhexan": "hexane", "n-hexan": "hexane",
            "nhexane": "hexane", "n-hexane": "hexane", "tetrahydrofuran": "thf", "h2o": "water",
            "dichlormethane": "ch2cl2"}
_GBSA_NAME = {"water": "h2o", "hexane": "nhexan"}


def data():
    global _DATA
    if _DATA is None:
        with open(_JSON) as f:
            _DATA = json.load(f)
    return _DATA


def parameter_set(solvent, kernel):
    """The GFN2 parameter set for `solvent`: GBSA sets for the Still kernel, ALPB sets for P16."""
    name = _ALIASES.get(solvent.lower(), solvent.lower())
    d = data()
    if kernel == "still":
        p = d["gbsa"].get(_GBSA_NAME.get(name, name))
    else:
        p = d["alpb"].get(name)
    if p is None:
        raise KeyError(f"solvent: '{name}' is not parametrized")
    return p


def lebedev_grid(nang):
    """Points (n, 3) and weights (n) of the Lebedev-Laikov grid the reference picks for `nang`.

    The grid index is the bisection of src/mctc/search.f90:37-79 over the 32 sizes: the largest
    size <= nang, except that nang equal to the largest size selects the one below it.
    """
    d = data()
    sizes = d["lebedev_sizes"]
    if nang < sizes[0]:
        raise ValueError("angular grid too small")
    if nang == sizes[-1]:
        size = sizes[-2]
    else:
        size = max(s for s in sizes if s <= nang)
    pts, wts = [], []
    for kind, a, b, v in d["lebedev"][str(size)]:
        kind = int(kind)
        if kind == 1:
            base = (1.0, 0.0, 0.0)
        elif kind == 2:
            base = (0.0, np.sqrt(0.5), np.sqrt(0.5))
        elif kind == 3:
            s = np.sqrt(1.0 / 3.0)
            base = (s, s, s)
        elif kind == 4:
            base = (a, a, np.sqrt(1.0 - 2.0 * a * a))
        elif kind == 5:
            base = (a, np.sqrt(1.0 - a * a), 0.0)
        else:
            base = (a, b, np.sqrt(1.0 - a * a - b * b))
        orbit = set()
        for perm in itertools.permutations(base):
            for signs in itertools.product((1.0, -1.0), repeat=3):
                orbit.add(tuple(s * x for s, x in zip(signs, perm)))
        orbit = sorted(orbit)
        pts.extend(orbit)
        wts.extend([v] * len(orbit))
    pts = np.array(pts)
    if len(pts) != size:
        raise ValueError(f"Lebedev grid {size}: {len(pts)} points")
    return pts, np.array(wts)


def state_shift(state, temperature, density, molar_mass):
    """Free-energy shift of the solution state, src/solv/state.f90."""
    if state == STATE_REFERENCE:
        return temperature * KB * (np.log(24.79 * temperature / 298.15) + np.log(density / 1.0e-3 * 1.0 / molar_mass))
    if state == STATE_MOL1BAR:
        return temperature * KB * np.log(24.79 * temperature / 298.15)
    return 0.0


class Solvation:
    """The generalised-Born + SASA model of one molecule (TBorn, src/solv/gbsa.f90)."""

    def __init__(self, Z, solvent, model="gbsa", kernel=None, alpb=None, nang=230, state=STATE_GSOLV,
                 temperature=298.15, ion_strength=0.0, ion_rad=0.0):
        Z = np.asarray(Z, dtype=np.int64)
        # xtb_setSolvent (src/api/calculator.f90:408-419): "gbsa" -> Still kernel, "alpb" -> ALPB
        # correction with the P16 kernel
        if kernel is None:
            kernel = "still" if model == "gbsa" else "p16"
        if alpb is None:
            alpb = model == "alpb"
        self.kernel = kernel
        p = parameter_set(solvent, kernel)
        d = data()
        eps = p["epsv"]
        self.eps = eps
        self.alpbet = ALPB_ALPHA / eps if alpb else 0.0
        self.keps = (1.0 / eps - 1.0) / (1.0 + self.alpbet)
        zi = Z - 1
        vdw = np.array(d["vdw_rad_d3"])[zi]
        sx = np.array(p["sx"])[zi]
        self.vdwr = vdw
        self.rho = vdw * sx
        self.svdw = vdw - p["soset"] * 0.1 * AATOAU
        self.c1 = p["c1"]
        self.vdwsa = vdw + p["rprobe"] * AATOAU
        self.trj2lo = (self.vdwsa - W) ** 2
        self.trj2hi = (self.vdwsa + W) ** 2

        def wpart(r):
            return (0.25 / W + 3.0 * AH3 * (0.2 * r * r - 0.5 * r * self.vdwsa + self.vdwsa ** 2 / 3.0)) * r ** 3

        self.wrp = wpart(self.vdwsa + W) - wpart(self.vdwsa - W)
        self.gamsasa = np.array(p["gamscale"])[zi] * 4.0 * PI * SURFACE_TENSION
        self.srcut = 2.0 * (W + np.max(self.vdwsa)) + ROFFSET
        tmp = np.array(p["tmp"])
        hb = -(tmp ** 2) * KCALTOAU if np.any(np.abs(tmp) > 1.0e-3) else np.zeros(94)
        self.hbmag = hb[zi]
        self.lhb = bool(np.any(self.hbmag < 0.0))
        density = p["rhos"] / p["smass"] * MOLCM3TOAU
        self.gshift = p["gshift"] * KCALTOAU + state_shift(state, temperature, density, p["smass"])
        self.grid, self.gw = lebedev_grid(nang)
        self.lsalt = ion_strength > 0.0
        if self.lsalt:
            self.kappa = 1.0 / (np.sqrt(eps * temperature * KAPPA_CONST / ion_strength) * AATOAU)
            self.ion_rad = ion_rad
        self.Z = Z

    # -- geometry-dependent part (TBorn%update, src/solv/gbsa.f90:392-442) -------------------
    def update(self, xyz):
        xyz = np.asarray(xyz, dtype=float).reshape(-1, 3)
        n = len(xyz)
        self.xyz = xyz
        d = xyz[:, None, :] - xyz[None, :, :]          # d[i, j] = x_i - x_j
        r = np.sqrt(np.sum(d * d, axis=2))
        self.d, self.r = d, r
        self._born_radii()
        self._sasa()
        self.gsasa = float(self.sasa @ self.gamsasa)
        if self.lsalt:
            aa = 0.5 / self.eps
            gg = self.kappa * (self.brad + self.ion_rad)
            self.ionscr = aa * np.exp(gg) / (1.0 + gg)
            self.discr = self.ionscr * self.kappa * gg / (1.0 + gg)
        if self.lhb:
            self.hbw = self.hbmag * self.sasa / self.vdwsa ** 2
            self.dhbdw = self.hbmag / self.vdwsa ** 2
        if self.alpbet > 0.0:
            self.adet = self._adet()
        self.B = self._born_matrix()
        return self

    def _pair_g(self):
        """psi contribution g[i, j] that atom j gives atom i, and dg = (dg/dr) / r."""
        n = len(self.Z)
        r = self.r.copy()
        np.fill_diagonal(r, 1.0)
        rhoj = np.broadcast_to(self.rho[None, :], (n, n))
        rvdwi = np.broadcast_to(self.vdwr[:, None], (n, n))
        ap, am = r + rhoj, r - rhoj
        overlap = r < rvdwi + rhoj
        with np.errstate(divide="ignore", invalid="ignore"):
            # separated spheres
            ab = ap * am
            rhab = rhoj / ab
            lnab = 0.5 * np.log(am / ap) / r
            g0 = rhab + lnab
            dg0 = -2.0 * rhab / ab + (rhab - lnab) / r ** 2
            # j's descreening sphere cuts i's van der Waals sphere
            r12 = 0.5 / r
            rh1 = 1.0 / rvdwi
            rhr1 = 1.0 / ap
            aprh1 = ap * rh1
            lnab1 = np.log(aprh1)
            g1 = rh1 - rhr1 + r12 * (0.5 * am * (rhr1 - rh1 * aprh1) - lnab1)
            dg1 = (rhr1 * rhr1 * (1.0 - 0.25 * am / r * (1.0 + aprh1 * aprh1))
                   + rhoj * r12 * r12 * (rhr1 - rh1 * aprh1) + r12 * (lnab1 / r - rhr1)) / r
        cut = (self.r < LRCUT) & ~np.eye(n, dtype=bool)
        part = overlap & (ap > rvdwi)
        g = np.where(cut & ~overlap, g0, np.where(cut & part, g1, 0.0))
        dg = np.where(cut & ~overlap, dg0, np.where(cut & part, dg1, 0.0))
        return g, dg

    def _born_radii(self):
        g, dg = self._pair_g()
        psi = g.sum(axis=1)
        s2 = 0.5 * self.svdw
        br = psi * s2
        arg2 = br * (OBC_GAMMA * br - OBC_BETA)
        arg = br * (OBC_ALPHA + arg2)
        darg = 2.0 * arg2 + OBC_ALPHA + OBC_GAMMA * br * br
        th, ch = np.tanh(arg), np.cosh(arg)
        den = 1.0 / self.svdw - th / self.vdwr
        self.brad = self.c1 / den
        self.dbrad = self.c1 * s2 / self.vdwr * darg / (ch * den) ** 2     # d brad / d psi
        self.psi, self.dg = psi, dg

    def _sasa(self):
        n = len(self.Z)
        sasa = np.zeros(n)
        ds = np.zeros((n, n, 3))                      # ds[i, k] = d sasa_i / d x_k
        self.sasap = np.zeros((n, len(self.gw)))
        for i in range(n):
            nb = np.nonzero((self.r[i] < self.srcut) & (np.arange(n) != i))[0]
            pts = self.xyz[i] + self.vdwsa[i] * self.grid               # [P, 3]
            tj = pts[:, None, :] - self.xyz[nb][None, :, :]              # [P, K, 3]
            tj2 = np.sum(tj * tj, axis=2)
            inside = tj2 < self.trj2hi[nb][None, :]
            buried = np.any(inside & (tj2 <= self.trj2lo[nb][None, :]), axis=1)
            sw = inside & ~(tj2 <= self.trj2lo[nb][None, :])
            sq = np.sqrt(tj2)
            uj = sq - self.vdwsa[nb][None, :]
            f = np.clip(AH0 + (AH1 + AH3 * uj * uj) * uj, 0.0, 1.0)
            df = AH1 + 3.0 * AH3 * uj * uj
            fsw = np.where(sw, f, 1.0)
            dead = buried | np.any(sw & (f < TINY), axis=1)
            sp = np.where(dead, 0.0, np.prod(fsw, axis=1))
            self.sasap[i] = sp
            live = sp > TOLSESP
            wsa = np.where(live, self.gw * self.wrp[i] * sp, 0.0)
            sasa[i] = np.sum(wsa)
            with np.errstate(divide="ignore", invalid="ignore"):
                gfac = np.where(sw & live[:, None], df / (f * sq), 0.0)
            dr = (wsa[:, None] * gfac)[:, :, None] * tj                  # [P, K, 3]
            contrib = dr.sum(axis=0)                                     # [K, 3]
            ds[i, i] += contrib.sum(axis=0)
            ds[i, nb] -= contrib
        self.sasa, self.dsasa = sasa, ds

    def _adet(self):
        x = self.xyz
        r3 = self.vdwr ** 3
        tot = r3.sum()
        c = (x * r3[:, None]).sum(axis=0) / tot
        v = x - c
        r2 = np.sum(v * v, axis=1)
        inertia = np.eye(3) * np.sum(r3 * (r2 + 0.4 * self.vdwr ** 2)) - np.einsum("a,ai,aj->ij", r3, v, v)
        self.inertia, self.center, self.totrad3 = inertia, c, tot
        return np.sqrt(np.linalg.det(inertia) ** (1.0 / 3.0) / (0.4 * tot))

    def _born_matrix(self):
        n = len(self.Z)
        a = self.brad
        r = self.r
        off = ~np.eye(n, dtype=bool)
        aa = a[:, None] * a[None, :]
        if self.lsalt:
            fgb = np.sqrt(r * r + aa * np.exp(-0.25 * r * r / aa))
            gg = self.ionscr[:, None] + self.ionscr[None, :]
            B = np.where(off, (np.exp(-self.kappa * fgb) * gg - 1.0) / fgb, 0.0)
            B += np.diag((np.exp(-self.kappa * a) * 2.0 * self.ionscr - 1.0) / a)
        elif self.kernel == "still":
            B = np.where(off, self.keps / np.sqrt(r * r + aa * np.exp(-0.25 * r * r / aa)), 0.0)
            B += np.diag(self.keps / a)
        else:
            ab = np.sqrt(aa)
            arg = (ab / (ab + ZETA_P16 / 16.0 * r)) ** 16
            B = np.where(off, self.keps / (r + ab * arg), 0.0)
            B += np.diag(self.keps / a)
        if self.lhb:
            B += np.diag(2.0 * self.hbw)
        if self.alpbet > 0.0:
            B += self.keps * self.alpbet / self.adet
        return B

    # -- SCC-time quantities ----------------------------------------------------------------
    def shift(self, q):
        return self.B @ q

    def energy(self, q):
        return 0.5 * float(q @ (self.B @ q)) + self.gsasa + self.gshift

    def energy_parts(self, q):
        """(G_born, G_hb, G_sasa, G_shift), getEnergyParts src/solv/gbsa.f90:552-596."""
        ghb = float(np.sum(self.hbw * q * q)) if self.lhb else 0.0
        return 0.5 * float(q @ (self.B @ q)) - ghb, ghb, self.gsasa, self.gshift

    def gradient(self, q):
        q = np.asarray(q, dtype=float)
        n = len(q)
        a = self.brad
        d, r = self.d, self.r
        off = ~np.eye(n, dtype=bool)
        rr = np.where(off, r, 1.0)
        qq = q[:, None] * q[None, :]
        aa = a[:, None] * a[None, :]
        grad = np.zeros((n, 3))
        if self.lsalt:
            dd = 0.25 * rr * rr / aa
            expd = np.exp(-dd)
            fgb2 = rr * rr + aa * expd
            fgb = np.sqrt(fgb2)
            ka = self.kappa * fgb
            expa = np.exp(-ka)
            gg = (self.ionscr[:, None] + self.ionscr[None, :]) * expa
            qfg = qq / fgb
            dfgb3 = qfg * (gg * (1.0 + ka) - 1.0) / fgb2
            ap = np.where(off, (1.0 - 0.25 * expd) * dfgb3, 0.0)
            bp = -0.5 * expd * (1.0 + dd) * dfgb3
            grddb = np.sum(np.where(off, a[None, :] * bp + qfg * expa * self.discr[:, None], 0.0), axis=1)
            ga = np.exp(-self.kappa * a)
            sa = 2.0 * self.ionscr * ga - 1.0
            apd = sa - a * 2.0 * (self.discr + self.ionscr * self.kappa) * ga
            grddb += -0.5 * (q / a) ** 2 * apd
            grad -= np.einsum("ij,ijk->ik", ap, d)
        elif self.kernel == "still":
            dd = 0.25 * rr * rr / aa
            expd = np.exp(-dd)
            dfgb = 1.0 / np.sqrt(rr * rr + aa * expd)
            dfgb3 = dfgb ** 3 * self.keps
            ap = np.where(off, (1.0 - 0.25 * expd) * dfgb3 * qq, 0.0)
            bp = np.where(off, -0.5 * expd * (1.0 + dd) * dfgb3 * qq, 0.0)
            grddb = bp @ a
            grddb += -0.5 * self.keps * q * q / (a * a)
            grad -= np.einsum("ij,ijk->ik", ap, d)
        else:
            ab = np.sqrt(aa)
            arg1 = ab / (ab + ZETA_P16 / 16.0 * rr)
            arg16 = arg1 ** 16
            dfgb = 1.0 / (rr + ab * arg16)
            ap = np.where(off, (1.0 - ZETA_P16 * arg1 * arg16) * dfgb ** 2 * self.keps / rr * qq, 0.0)
            bp = np.where(off, -0.5 * (rr * ZETA_P16 / ab * arg1 + 1.0) / ab * arg16 * dfgb ** 2 * self.keps * qq, 0.0)
            grddb = bp @ a
            grddb += -0.5 * self.keps * q * q / (a * a)
            grad -= np.einsum("ij,ijk->ik", ap, d)
        # Born radii chain: d brad_i / d x_k through psi_i
        wgt = grddb * self.dbrad
        pair = wgt[:, None] * self.dg + (wgt[:, None] * self.dg).T      # w_k dg_k(j) + w_j dg_j(k)
        grad += np.einsum("kj,kjc->kc", pair, d)
        # surface term and hydrogen-bond correction
        wsur = self.gamsasa.copy()
        if self.lhb:
            wsur = wsur + self.dhbdw * q * q
        grad += np.einsum("i,ikc->kc", wsur, self.dsasa)
        # ALPB shape term (vanishes for neutral molecules)
        if self.alpbet > 0.0:
            qt = float(np.sum(q))
            I3, adet, tot = self.inertia, self.adet, self.totrad3
            M = np.array([
                [I3[0, 0] * (I3[1, 1] + I3[2, 2]) - I3[0, 1] ** 2 - I3[0, 2] ** 2,
                 I3[0, 1] * I3[2, 2] - I3[0, 2] * I3[1, 2], I3[0, 2] * I3[1, 1] - I3[0, 1] * I3[2, 1]],
                [I3[0, 1] * I3[2, 2] - I3[0, 2] * I3[1, 2],
                 I3[1, 1] * (I3[0, 0] + I3[2, 2]) - I3[0, 1] ** 2 - I3[1, 2] ** 2,
                 I3[0, 0] * I3[1, 2] - I3[0, 1] * I3[0, 2]],
                [I3[0, 2] * I3[1, 1] - I3[0, 1] * I3[2, 1], I3[0, 0] * I3[1, 2] - I3[0, 1] * I3[0, 2],
                 I3[2, 2] * (I3[0, 0] + I3[1, 1]) - I3[0, 2] ** 2 - I3[1, 2] ** 2]])
            M = M * (250.0 / (48.0 * tot ** 3 * adet ** 5)) * (-0.5 * self.keps * self.alpbet * qt ** 2 / adet ** 2)
            v = self.xyz - self.center
            grad += (self.vdwr ** 3)[:, None] * (v @ M.T)
        return grad
