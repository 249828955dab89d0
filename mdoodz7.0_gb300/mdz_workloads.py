"""Seeded synthetic workloads for the local rheology update.

MDOODZ7.0 measures this path only inside full simulations; there is no public
dataset.  These generators build `grid`-shaped inputs with the shapes, sizes
and value distributions of the five benchmark workloads:

  * ``plain_small``   201 x 201 cells, 2 phases (dislocation creep + elasticity
                      + Drucker-Prager), the CPU-runnable case;
  * ``plain_large``   2049 x 2049 cells, 5 phases mixing dislocation,
                      diffusion and Peierls creep with softened plasticity;
  * ``multi_grid``    64 grids of uneven size (65^2 .. 1025^2 cells);
  * ``aniso``         anisotropic variant (director angle, anisotropy factor).

Material tables follow MDOODZ7.0's unit and correction conventions
(MDLIB/FlowLaws.c:46-589 power-law database, correction factor F for the
invariant formulation at MDLIB/FlowLaws.c:572-575, scaling at
MDLIB/InputOutput.c:1835-1849); with the default SI scaling (all scales 1)
values are used as written.  Strain-softened friction is computed exactly like
`Softening` style 0 with arithmetic phase averaging
(MDLIB/RheologyDensity.c:1432-1532).

All randomness comes from numpy's PCG64 generator, so a seed gives the same
fields on every host.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

import mdz_rheo as R

RG = 8.314510        # MDLIB/include/mdoodz.h:5
ZEROC = 273.15       # MDLIB/include/mdoodz.h:4
DEG = math.pi / 180.0


# ---- scaling -----------------------------------------------------------------
@dataclass
class Scale:
    """Characteristic scales of `scale` (MDLIB/include/mdoodz.h:142-144), derived
    from eta, L, V, T the way ScaleMe does (MDLIB/InputOutput.c:1835-1849)."""
    eta: float = 1.0
    L: float = 1.0
    V: float = 1.0
    T: float = 1.0

    @property
    def t(self):
        return self.L / self.V

    @property
    def E(self):
        return 1.0 / self.t

    @property
    def S(self):
        return self.eta / self.t

    @property
    def J(self):
        return self.S * self.L ** 3

    @property
    def rho(self):
        return self.S * self.t ** 2 / self.L ** 2


SI = Scale()
# A typical MDOODZ setup scaling (SETS/*.txt: eta=1e20, L=1e4, V=1e-9, T=600)
TYPICAL = Scale(eta=1e20, L=1e4, V=1e-9, T=600.0)


# ---- materials -----------------------------------------------------------------
def correction_factor(t: float, n: float) -> float:
    """Invariant-formulation correction F (MDLIB/FlowLaws.c:572-575)."""
    if t == 0:
        return 1.0
    if t == 1:
        return 1.0 / 6.0 * math.pow(2.0, 1.0 / n) * math.pow(3.0, (n - 1.0) / 2.0 / n)
    if t == 2:
        return 1.0 / 4 * math.pow(2.0, 1.0 / n)
    raise ValueError(t)


def empty_materials(nphases: int, sc: Scale = SI) -> R.Materials:
    """Defaults of ReadInputFile's material block (MDLIB/InputOutput.c:1368-1451)."""
    m = R.Materials()
    m.Nb_phases = nphases
    m.R = RG / (sc.J / sc.T)
    for p in range(R.MAX_PHASES):
        m.rho[p] = 2700.0 / sc.rho
        m.bet[p] = 1e-40 * sc.S
        m.T0[p] = ZEROC / sc.T
        m.P0[p] = 1e5 / sc.S
        m.plast[p] = 1
        m.T_st[p] = -10.0e6 / sc.S
        m.Slim[p] = 1.0e90 / sc.S
        m.n_vp[p] = 1.0
        m.eta_vp[p] = 0.0
        m.eta0[p] = 1.0e20 / sc.eta
        m.npwl[p] = 1.0
        m.pref_pwl[p] = 1.0
        m.gs_ref[p] = 2.0e-3 / sc.L
        m.density_model[p] = 3
        m.nlin[p] = 1.0
        m.ngbs[p] = 1.0
        m.Fpwl[p] = m.Flin[p] = m.Fgbs[p] = 1.0
    return m


def set_power_law(m: R.Materials, p: int, A: float, n: float, Q: float, V: float, t: int = 1,
                  mexp: float = 0.0, r: float = 0.0, f: float = 0.0, a: float = 0.0,
                  sc: Scale = SI):
    """Dislocation creep entry with ReadDataPowerLaw's scaling (MDLIB/FlowLaws.c:561-575)."""
    m.pwlv[p] = 1
    m.npwl[p] = n
    m.mpwl[p] = mexp
    m.rpwl[p] = r
    m.Qpwl[p] = Q / sc.J
    m.Vpwl[p] = V / sc.L ** 3
    m.Apwl[p] = A / (sc.S ** (-n) * sc.S ** (-r) * sc.L ** mexp / sc.t)
    m.fpwl[p] = f / sc.S
    m.apwl[p] = a
    m.Fpwl[p] = correction_factor(t, n)


def set_linear(m: R.Materials, p: int, A: float, n: float, mexp: float, Q: float, V: float,
               t: int = 1, sc: Scale = SI):
    """Diffusion creep entry (MDLIB/FlowLaws.c:591-700)."""
    m.linv[p] = 1
    m.nlin[p] = n
    m.mlin[p] = mexp
    m.rlin[p] = 0.0
    m.Qlin[p] = Q / sc.J
    m.Vlin[p] = V / sc.L ** 3
    m.Alin[p] = A / (sc.S ** (-n) * sc.L ** mexp / sc.t)
    m.flin[p] = 0.0
    m.alin[p] = 0.0
    m.Flin[p] = correction_factor(t, n)


def set_peierls(m: R.Materials, p: int, Q=5.4e5, S=8.5e9, E=5.7e11, G=0.1, n=0.0, sc: Scale = SI):
    """Regularised Peierls creep (MDLIB/FlowLaws.c:807-842)."""
    m.expv[p] = 1
    m.Qexp[p] = Q / sc.J
    m.Sexp[p] = S / sc.S
    m.Eexp[p] = E / (sc.E * sc.S ** (-n))
    m.Gexp[p] = G
    m.nexp[p] = n


# The five flow-law phases of the large plain workload.  Each tuple is
# (dislocation law or None, diffusion?, Peierls?).
OLIVINE_DRY = dict(A=1.1e-16, n=3.5, Q=530e3, V=11e-6, t=1)            # FlowLaws.c:457-470
SOFT_QTZ = dict(A=5.1e-4 * 10.0 ** (-6 * 2.3), n=2.3, Q=154e3, V=0.0, t=1)  # 5.1e-4 MPa^-n/s
OLIVINE_DIFF = dict(A=1.5e-15, n=1.0, mexp=3.0, Q=375e3, V=4e-6, t=1)    # FlowLaws.c:651-664
PEIERLS = dict(Q=5.4e5, S=5.9e9, E=5.7e11, G=0.1, n=0.0)                # FlowLaws.c:807-817, sigma_P=5.9e9

PLAIN_LARGE_PHASES = [
    ("olivine: dislocation+diffusion+Peierls", OLIVINE_DRY, True, True),
    ("soft quartz: dislocation", SOFT_QTZ, False, False),
    ("fine-grained: diffusion only", None, True, False),
    ("olivine: dislocation+Peierls", OLIVINE_DRY, False, True),
    ("soft quartz + diffusion", SOFT_QTZ, True, False),
]


def materials_plain_small(sc: Scale = SI) -> R.Materials:
    m = empty_materials(2, sc)
    set_power_law(m, 0, sc=sc, **OLIVINE_DRY)
    set_power_law(m, 1, sc=sc, **SOFT_QTZ)
    return m


def materials_plain_large(nphases: int = 5, sc: Scale = SI, phase_ids: Optional[List[int]] = None
                          ) -> R.Materials:
    ids = list(range(nphases)) if phase_ids is None else phase_ids
    m = empty_materials(len(ids), sc)
    for p, k in enumerate(ids):
        _, pwl, lin, pei = PLAIN_LARGE_PHASES[k]
        if pwl is not None:
            set_power_law(m, p, sc=sc, **pwl)
        if lin:
            set_linear(m, p, sc=sc, **OLIVINE_DIFF)
        if pei:
            set_peierls(m, p, sc=sc, **PEIERLS)
    return m


def make_model(ncx: int, ncz: int, nphases: int, dt: float = 1e11, sc: Scale = SI,
               eta_average: int = 0) -> R.Model:
    md = R.Model()
    md.Nx, md.Nz, md.Nb_phases = ncx + 1, ncz + 1, nphases
    md.step, md.elastic, md.eta_average = 1, 1, eta_average
    md.periodic_x, md.density_variations, md.tensile_line_search = 0, 0, 0
    md.melting = md.chemical_production = md.diffuse_X = md.diffuse_avg = 0
    md.dt = dt / sc.t
    md.min_eta, md.max_eta = 1e18 / sc.eta, 1e25 / sc.eta
    md.eta_tol = 1e-11  # set explicitly; ReadInputFile's default is 1e11 (InputOutput.c:1205)
    md.scale_eta, md.scale_L, md.scale_T, md.scale_S, md.scale_E = sc.eta, sc.L, sc.T, sc.S, sc.E
    return md


# ---- fields --------------------------------------------------------------------
def smooth_fields(rng, nfields, xs, zs, modes=6, kmax=3):
    """`nfields` smooth random fields on the tensor grid xs x zs (coordinates in
    [0,1]): sums of `modes` low-wavenumber plane waves, unit variance."""
    out = np.zeros((nfields, zs.size, xs.size))
    for f in range(nfields):
        for _ in range(modes):
            kx, kz = rng.integers(-kmax, kmax + 1, size=2)
            ph = rng.uniform(0, 2 * np.pi)
            amp = rng.normal()
            ax = 2 * np.pi * kx * xs + ph
            az = 2 * np.pi * kz * zs
            # cos(ax + az) separably
            out[f] += amp * (np.outer(np.cos(az), np.cos(ax)) - np.outer(np.sin(az), np.sin(ax)))
        sd = out[f].std()
        if sd > 0:
            out[f] /= sd
    return out


def phase_fractions(g, sharp=3.0):
    """Softmax of smooth fields: positive, sum to 1 at every node."""
    e = np.exp(sharp * (g - g.max(axis=0, keepdims=True)))
    return e / e.sum(axis=0, keepdims=True)


def loguniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def signed_loguniform(rng, lo, hi, n):
    return loguniform(rng, lo, hi, n) * rng.choice([-1.0, 1.0], n)


@dataclass
class Workload:
    name: str
    model: R.Model
    mat: R.Materials
    arrays: Dict[str, object]
    info: Dict[str, object] = field(default_factory=dict)

    @property
    def Nc(self):
        return (self.model.Nx - 1) * (self.model.Nz - 1)

    @property
    def Nv(self):
        return self.model.Nx * self.model.Nz

    @property
    def nodes(self):
        return self.Nc + self.Nv


def alloc_outputs(arrays, nc, nv, nphases, aniso=False, density=False):
    for k in R.VER_INTERP:
        arrays[k] = np.zeros(nv)
    for k in R.CEN_OUT:
        if k == "rho_n" and not density:
            continue
        arrays[k] = np.zeros(nc)
    for k in R.VER_OUT:
        if k == "VE_s" and not aniso:
            continue
        arrays[k] = np.zeros(nv)
    arrays["phase_eta_n"] = [np.zeros(nc) for _ in range(nphases)]
    arrays["phase_eta_s"] = [np.zeros(nv) for _ in range(nphases)]


def grid_workload(name, ncx, ncz, mat: R.Materials, seed: int, dt=1e11, sc: Scale = SI,
                  grain_size=None, softening=None, aniso=False, strain_range=(0.0, 1.0),
                  eta_average=0, T_range=(500.0, 1400.0), depth=100e3,
                  Erange=(1e-16, 1e-13), stress=50e6) -> Workload:
    """Fill every input field of a (ncx x ncz)-cell grid from `seed`.

    T ~ U(T_range) at centroids; P = rho g z with rho=3000, g=9.81 and depth z
    linear in row index (row 0 deepest, top row 0 km) over `depth`; Exx=-Ezz
    and Exz log-uniform in magnitude over Erange with random sign, drawn
    independently at centroids and vertices; old deviatoric stresses
    sxxd0 ~ U(+-stress), szzd0=-sxxd0, sxz0 ~ U(+-stress); phase fractions
    are a softmax of smooth random fields; G=3e10, beta=1e-40, C=1e7,
    dilation 0, friction 30 deg (or softened: `softening` = (phi0_deg,
    phi_end_deg, pls_start, pls_end) with plastic strain ~ U(strain_range)).
    `grain_size` = (lo, hi) draws d log-uniformly, else d = 2 mm.
    """
    rng = np.random.default_rng(seed)
    nphases = mat.Nb_phases
    nx, nz = ncx + 1, ncz + 1
    nc, nv = ncx * ncz, nx * nz
    a: Dict[str, object] = {}
    # coordinates in [0,1]: centroids at cell middles, vertices at cell corners
    xc = (np.arange(ncx) + 0.5) / ncx
    zc = (np.arange(ncz) + 0.5) / ncz
    xv = np.arange(nx) / ncx
    zv = np.arange(nz) / ncz
    g_seed = rng.integers(1 << 62)
    gc = smooth_fields(np.random.default_rng(g_seed), nphases, xc, zc)
    gv = smooth_fields(np.random.default_rng(g_seed), nphases, xv, zv)
    pc = phase_fractions(gc).reshape(nphases, nc)
    pv = phase_fractions(gv).reshape(nphases, nv)
    a["phase_perc_n"] = [np.ascontiguousarray(pc[p]) for p in range(nphases)]
    a["phase_perc_s"] = [np.ascontiguousarray(pv[p]) for p in range(nphases)]
    # temperature and pressure
    T = rng.uniform(T_range[0], T_range[1], nc) / sc.T
    zdepth_c = depth * (1.0 - zc)               # row 0 deepest
    zdepth_v = depth * (1.0 - zv)
    Pc = np.repeat(3000.0 * 9.81 * zdepth_c, ncx) / sc.S
    Pv = np.repeat(3000.0 * 9.81 * zdepth_v, nx) / sc.S
    a["T"] = T
    a["p_in"] = Pc
    a["T0_n"] = T.copy()
    a["p0_n"] = Pc.copy()
    a["p0_s"] = Pv.copy()
    # strain rates and old stresses
    for suffix, n in (("n", nc), ("s", nv)):
        exx = signed_loguniform(rng, Erange[0], Erange[1], n) / sc.E
        exz = signed_loguniform(rng, Erange[0], Erange[1], n) / sc.E
        sxx0 = rng.uniform(-stress, stress, n) / sc.S
        sxz0 = rng.uniform(-stress, stress, n) / sc.S
        if suffix == "n":
            a["exxd"], a["ezzd"], a["exz_n"] = exx, -exx, exz
            a["sxxd0"], a["szzd0"], a["sxz0_n"] = sxx0, -sxx0, sxz0
        else:
            a["exxd_s"], a["ezzd_s"], a["exz"] = exx, -exx, exz
            a["sxxd0_s"], a["szzd0_s"], a["sxz0"] = sxx0, -sxx0, sxz0
    # grain size
    if grain_size is not None:
        a["d0_n"] = loguniform(rng, grain_size[0], grain_size[1], nc) / sc.L
    else:
        a["d0_n"] = np.full(nc, 2e-3 / sc.L)
    # plasticity inputs (Softening style 0, arithmetic average)
    for suffix, n, perc in (("n", nc, pc), ("s", nv, pv)):
        if softening is not None:
            phi0, phie, plss, plse = softening
            eps = rng.uniform(strain_range[0], strain_range[1], n)
            fr = np.where(eps < plss, phi0 * DEG,
                          np.where(eps >= plse, phie * DEG,
                                   phi0 * DEG + (phie * DEG - phi0 * DEG) / (plse - plss) * eps))
            fric = np.zeros(n)
            for p in range(nphases):
                fric += perc[p] * fr
        else:
            eps = np.zeros(n)
            fric = np.full(n, 30.0 * DEG)
        a["strain_" + suffix] = eps
        a["fric_" + suffix] = fric
        a["C_" + suffix] = np.full(n, 1e7 / sc.S)
        a["dil_" + suffix] = np.zeros(n)
        a["mu_" + suffix] = np.full(n, 3e10 / sc.S)
        a["bet_" + suffix] = np.full(n, 1e-40 * sc.S)
        a["X0_" + suffix] = np.zeros(n)
    a["phi0_n"] = np.zeros(nc)
    a["div_u"] = np.zeros(nc)
    a["div_u_s"] = np.zeros(nv)
    a["BCp_type"] = np.full(nc, -1, dtype=np.int8)
    a["BCg_type"] = np.full(nv, -1, dtype=np.int8)
    if aniso:
        for suffix, n in (("n", nc), ("s", nv)):
            th = rng.uniform(0.0, np.pi, n)
            delta = loguniform(rng, 1.0, 10.0, n)
            # director components as ParticleRoutines.c:1989-1998 / AnisotropyRoutines.c:1244-1245
            nx_, nz_ = np.cos(th), np.sin(th)
            a["d1_" + suffix] = 2.0 * nx_ ** 2 * nz_ ** 2
            a["d2_" + suffix] = nx_ * nz_ * (-nx_ ** 2 + nz_ ** 2)
            a["angle_" + suffix] = th
            a["aniso_factor_" + suffix] = delta
    alloc_outputs(a, nc, nv, nphases, aniso=aniso)
    model = make_model(ncx, ncz, nphases, dt=dt, sc=sc, eta_average=eta_average)
    return Workload(name, model, mat, a, info=dict(seed=seed, ncx=ncx, ncz=ncz, nphases=nphases))


def plain_small(seed: int = 0, ncx: int = 201, ncz: Optional[int] = None, sc: Scale = SI,
                eta_average: int = 0) -> Workload:
    """201 x 201 cells, 2 phases, dt = 1e11 s, cutoffs 1e18-1e25 Pa s."""
    ncz = ncx if ncz is None else ncz
    return grid_workload("plain_small", ncx, ncz, materials_plain_small(sc), seed, sc=sc,
                         eta_average=eta_average)


def plain_large(seed: int = 1, ncx: int = 2049, ncz: Optional[int] = None, sc: Scale = SI,
                nphases: int = 5, eta_average: int = 0) -> Workload:
    """2049 x 2049 cells, 5 phases (dislocation, diffusion with d log-U(1e-5,1e-2) m,
    Peierls with sigma_P=5.9e9 Pa, Drucker-Prager softened 30->5 deg over
    plastic strain U(0,1))."""
    ncz = ncx if ncz is None else ncz
    return grid_workload("plain_large", ncx, ncz, materials_plain_large(nphases, sc), seed, sc=sc,
                         grain_size=(1e-5, 1e-2), softening=(30.0, 5.0, 0.0, 1.0),
                         eta_average=eta_average)


def aniso(seed: int = 4, ncx: int = 4097, ncz: Optional[int] = None, sc: Scale = SI,
          nphases: int = 3) -> Workload:
    """Anisotropic workload: 3 phases with dislocation creep and DP as the large plain
    case, director angle U[0,pi), anisotropy factor log-U(1,10)."""
    ncz = ncx if ncz is None else ncz
    m = empty_materials(nphases, sc)
    laws = [OLIVINE_DRY, SOFT_QTZ, OLIVINE_DRY]
    for p in range(nphases):
        set_power_law(m, p, sc=sc, **laws[p % 3])
    return grid_workload("aniso", ncx, ncz, m, seed, sc=sc, softening=(30.0, 5.0, 0.0, 1.0),
                         aniso=True)


def many_grids(seed: int = 7, n: int = 64, lo: int = 65, hi: int = 1025, sc: Scale = SI) -> List[Workload]:
    """Many independent grids of uneven size for one batched launch: cells per side
    log-uniform in [lo, hi], 2-5 phases drawn from the large plain workload's five,
    dt log-uniform in 1e10-1e12 s, each grid with its own seed."""
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n):
        side = int(round(float(loguniform(rng, lo, hi, 1)[0])))
        nph = int(rng.integers(2, 6))
        ids = sorted(rng.choice(len(PLAIN_LARGE_PHASES), size=nph, replace=False).tolist())
        dt = float(loguniform(rng, 1e10, 1e12, 1)[0])
        mat = materials_plain_large(nph, sc, phase_ids=ids)
        out.append(grid_workload("many_grids", side, side, mat, seed * 1000 + g, dt=dt, sc=sc,
                                 grain_size=(1e-5, 1e-2), softening=(30.0, 5.0, 0.0, 1.0)))
    return out


def velocity_field(seed: int = 9, ncx: int = 2049, ncz: Optional[int] = None, air: float = 0.0,
                   periodic: int = 0, sc: Scale = SI, L: float = 1e5, v0: float = 1e-9) -> Workload:
    """Input of StrainRateComponents on ncx x ncz cells: staggered velocities of a smooth
    random flow, u at Nx x (Nz+1) nodes and v at (Nx+1) x Nz nodes (rows include the
    ghost nodes of MDOODZ's staggered grid), about v0 m/s plus 1 % node-scale noise, on a
    square L x L domain.  With air > 0 the top part of the domain above a wavy surface at
    height 1 - air (fraction of L) is air: those cells have BCp_type 30, those of the row
    just below the surface 31, vertices above it BCg_type 30.  Output arrays are filled
    with a sentinel (wxz keeps it at air vertices).  dx and dz are in `info`."""
    ncz = ncx if ncz is None else ncz
    rng = np.random.default_rng(seed)
    nx, nz = ncx + 1, ncz + 1
    nc, nv = ncx * ncz, nx * nz
    dx, dz = L / ncx / sc.L, L / ncz / sc.L
    vs = v0 / (sc.L / sc.t)

    def flow(xs, zs):
        f = smooth_fields(rng, 1, xs, zs)[0]
        return vs * (f + 0.01 * rng.standard_normal(f.shape))

    # u node (k, l): x = k / ncx, z = (l - 0.5) / ncz; v node (k, l): x = (k - 0.5) / ncx, z = l / ncz
    u = flow(np.arange(nx) / ncx, (np.arange(nz + 1) - 0.5) / ncz)
    v = flow((np.arange(nx + 1) - 0.5) / ncx, np.arange(nz) / ncz)
    a: Dict[str, object] = {"u_in": np.ascontiguousarray(u.ravel()), "v_in": np.ascontiguousarray(v.ravel())}
    bcp = np.full((ncz, ncx), -1, dtype=np.int8)
    bcg = np.full((nz, nx), -1, dtype=np.int8)
    if air > 0.0:
        ph = rng.uniform(0, 2 * np.pi)
        xc, zc = (np.arange(ncx) + 0.5) / ncx, (np.arange(ncz) + 0.5) / ncz
        h = 1.0 - air + 0.05 * np.sin(4.0 * np.pi * xc + ph)
        above = zc[:, None] > h[None, :]
        bcp[above] = 30
        below = (~above) & (zc[:, None] > h[None, :] - 1.0 / ncz)
        bcp[below] = 31
        xv, zv = np.arange(nx) / ncx, np.arange(nz) / ncz
        hv = 1.0 - air + 0.05 * np.sin(4.0 * np.pi * xv + ph)
        bcg[zv[:, None] > hv[None, :]] = 30
    a["BCp_type"] = bcp.ravel()
    a["BCg_type"] = bcg.ravel()
    for k in R.SR_N:
        a[k] = np.full(nc, -7.0)
    for k in R.SR_S:
        a[k] = np.full(nv, -7.0)
    model = make_model(ncx, ncz, 1, sc=sc)
    model.periodic_x = periodic
    return Workload("velocity_field", model, None, a, info=dict(seed=seed, ncx=ncx, ncz=ncz, dx=dx, dz=dz))


def logistic(x, top):
    """top / (1 + exp(-2x)), i.e. top (1 + tanh x) / 2, through exp, which numpy evaluates
    alike on x86 and Arm hosts (its tanh differs between them in the last bits)."""
    return top / (1.0 + np.exp(-2.0 * x))


def prep_materials(rng, nphases: int, sc: Scale = SI) -> R.PrepMaterials:
    """Per-phase constants of the sweep's input preparation (Softening and
    ShearModCompExpGrid): shear modulus 1e10-8e10 Pa, compressibility 1e-12-1e-10 1/Pa,
    expansivity 1e-5-4e-5 1/K, cohesion 1e6-5e7 Pa softening to 5-50 % of it, friction
    20-35 deg softening to 2-10 deg, dilation 0-10 deg softening to 0, softening between
    plastic strains U(0, 0.2) and that + U(0.3, 1), linear cohesion hardening -1e6..-1e7 Pa
    (negative: weakening), each softening switch on with probability 0.7."""
    m = R.PrepMaterials()
    m.Nb_phases = nphases
    for p in range(nphases):
        m.G[p] = float(loguniform(rng, 1e10, 8e10, 1)[0]) / sc.S
        m.bet[p] = float(loguniform(rng, 1e-12, 1e-10, 1)[0]) * sc.S
        m.alp[p] = float(rng.uniform(1e-5, 4e-5)) * sc.T
        m.C[p] = float(loguniform(rng, 1e6, 5e7, 1)[0]) / sc.S
        m.C_end[p] = m.C[p] * float(rng.uniform(0.05, 0.5))
        m.phi[p] = float(rng.uniform(20.0, 35.0)) * DEG
        m.phi_end[p] = float(rng.uniform(2.0, 10.0)) * DEG
        m.psi[p] = float(rng.uniform(0.0, 10.0)) * DEG
        m.psi_end[p] = 0.0
        m.pls_start[p] = float(rng.uniform(0.0, 0.2))
        m.pls_end[p] = m.pls_start[p] + float(rng.uniform(0.3, 1.0))
        m.H_c[p] = -float(loguniform(rng, 1e6, 1e7, 1)[0]) / sc.S
        m.phi_soft[p], m.psi_soft[p], m.coh_soft[p] = [int(x) for x in rng.random(3) < 0.7]
    return m


def prep_workload(seed: int = 13, ncx: int = 2049, ncz: Optional[int] = None, nphases: int = 5, air: float = 0.0,
                  periodic: int = 0, markers_per_cell: int = 0, sc: Scale = SI, L: float = 1e5) -> Workload:
    """Input of the sweep's preparation steps on ncx x ncz cells: phase fractions from
    smooth random fields (softmax, fractions below 3 % set to exactly zero and the rest
    renormalised, as marker interpolation leaves many exact zeros), plastic strain from a
    smooth field in [0, 1.5) with 1 % of the nodes exactly at phase 0's pls_start and 1 %
    at its pls_end, marker noise U(-0.1, 0.1), air above a wavy surface as in
    velocity_field.  With markers_per_cell > 0, `info["markers"]` also holds that many
    markers per cell at uniform random positions (phase and plastic strain attached) on an
    L x L domain, for the reference's own marker-to-grid interpolation."""
    ncz = ncx if ncz is None else ncz
    rng = np.random.default_rng(seed)
    nx, nz = ncx + 1, ncz + 1
    nc, nv = ncx * ncz, nx * nz
    pm = prep_materials(rng, nphases, sc)
    xc, zc = (np.arange(ncx) + 0.5) / ncx, (np.arange(ncz) + 0.5) / ncz
    xv, zv = np.arange(nx) / ncx, np.arange(nz) / ncz
    a: Dict[str, object] = {}
    for suffix, xs, zs in (("n", xc, zc), ("s", xv, zv)):
        frac = phase_fractions(smooth_fields(rng, nphases, xs, zs)).reshape(nphases, -1)
        frac[frac < 0.03] = 0.0
        frac /= frac.sum(axis=0, keepdims=True)
        a["phase_perc_" + suffix] = [np.ascontiguousarray(frac[p]) for p in range(nphases)]
        st = logistic(smooth_fields(rng, 1, xs, zs)[0], 1.5).ravel()
        k = rng.permutation(st.size)
        st[k[: st.size // 100]] = pm.pls_start[0]
        st[k[st.size // 100: st.size // 50]] = pm.pls_end[0]
        a["strain_pl_" + suffix] = st
        a["noise_" + suffix] = rng.uniform(-0.1, 0.1, st.size)
    bcp = np.full((ncz, ncx), -1, dtype=np.int8)
    bcg = np.full((nz, nx), -1, dtype=np.int8)
    if air > 0.0:
        ph = rng.uniform(0, 2 * np.pi)
        h = 1.0 - air + 0.05 * np.sin(4.0 * np.pi * xc + ph)
        above = zc[:, None] > h[None, :]
        bcp[above] = 30
        bcp[(~above) & (zc[:, None] > h[None, :] - 1.0 / ncz)] = 31
        hv = 1.0 - air + 0.05 * np.sin(4.0 * np.pi * xv + ph)
        bcg[zv[:, None] > hv[None, :]] = 30
    a["BCp_type"], a["BCg_type"] = bcp.ravel(), bcg.ravel()
    for k in R.SOFT_N + R.MOD_N:
        a[k] = np.full(nc, -7.0)
    for k in R.SOFT_S + R.MOD_S:
        a[k] = np.full(nv, -7.0)
    model = make_model(ncx, ncz, nphases, sc=sc)
    model.periodic_x = periodic
    info = dict(seed=seed, ncx=ncx, ncz=ncz)
    if markers_per_cell > 0:
        n = nc * markers_per_cell
        dx, dz = L / ncx / sc.L, L / ncz / sc.L
        x = rng.uniform(0.0, ncx * dx, n)
        z = rng.uniform(0.0, ncz * dz, n)
        phase = rng.integers(0, nphases, n).astype(np.int32)
        g = smooth_fields(rng, 1, np.linspace(0, 1, 64), np.linspace(0, 1, 64))[0]
        ix = np.minimum((x / (ncx * dx) * 64).astype(int), 63)
        iz = np.minimum((z / (ncz * dz) * 64).astype(int), 63)
        strain = logistic(g[iz, ix], 1.5) * rng.uniform(0.8, 1.2, n)
        info["markers"] = dict(x=x, z=z, phase=phase, strain_pl=strain, xmin=0.0, zmin=0.0, dx=dx, dz=dz,
                               interp_stencil=1)
    return Workload("prep", model, pm, a, info=info)


def marker_workload(seed: int = 17, ncx: int = 2049, ncz: Optional[int] = None, markers_per_cell: int = 4,
                    air: float = 0.0, periodic: int = 0, inactive: float = 0.02, sc: Scale = SI,
                    L: float = 1e5) -> Workload:
    """Input of UpdateParticleStress on ncx x ncz cells of an L x L domain at x in
    [-L/2, L/2], z in [-L, 0]: node coordinates built as the reference builds them
    (running sums of dx from xmin, GridRoutines.c:270-315), the sweep's new and old
    deviatoric stresses (normal, 10 MPa spread, with increments of 1 %), smooth random
    velocities as in velocity_field, a spin field wxz to be overwritten, and markers
    per cell at uniform random positions with random stresses and unit directors, a
    fraction `inactive` of them with phase -1, laid out cell by cell as MDOODZ seeds them.
    Air above a wavy surface as in velocity_field.  `arrays` holds the grid fields, `info` the
    markers, dx, dz and the per-phase shear modulus G."""
    ncz = ncx if ncz is None else ncz
    rng = np.random.default_rng(seed)
    nx, nz = ncx + 1, ncz + 1
    nc, nv = ncx * ncz, nx * nz
    dx, dz = L / ncx / sc.L, L / ncz / sc.L
    xmin, zmin = -0.5 * L / sc.L, -L / sc.L

    def running(x0, step, n):
        out = np.empty(n)
        out[0] = x0
        for i in range(1, n):
            out[i] = out[i - 1] + step
        return out

    a: Dict[str, object] = {"xg_coord": running(xmin, dx, nx), "zg_coord": running(zmin, dz, nz),
                            "xvz_coord": running(xmin - dx / 2.0, dx, nx + 1),
                            "zvx_coord": running(zmin - dz / 2.0, dz, nz + 1)}
    S = 1e7 / sc.S
    a["sxxd"], a["szzd"] = S * rng.standard_normal(nc), S * rng.standard_normal(nc)
    a["sxxd0"] = a["sxxd"] * (1.0 + 0.01 * rng.standard_normal(nc))
    a["szzd0"] = a["szzd"] * (1.0 + 0.01 * rng.standard_normal(nc))
    a["sxz"] = S * rng.standard_normal(nv)
    a["sxz0"] = a["sxz"] * (1.0 + 0.01 * rng.standard_normal(nv))
    vel = velocity_field(seed=seed + 1, ncx=ncx, ncz=ncz, air=air, periodic=periodic, sc=sc, L=L)
    for k in ("u_in", "v_in", "BCp_type", "BCg_type"):
        a[k] = vel.arrays[k]
    a["wxz"] = rng.standard_normal(nv) * 1e-14 * sc.t
    n = nc * markers_per_cell
    phase = rng.integers(0, 3, n).astype(np.int32)
    phase[rng.random(n) < inactive] = -1
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    # cell by cell, as MDOODZ seeds them (uniform within each cell)
    cell = np.repeat(np.arange(nc), markers_per_cell)
    mk = {"x": xmin + ((cell % ncx) + rng.random(n)) * dx, "z": zmin + ((cell // ncx) + rng.random(n)) * dz,
          "phase": phase,
          "sxxd": S * rng.standard_normal(n), "szzd": S * rng.standard_normal(n), "sxz": S * rng.standard_normal(n),
          "nx": np.cos(th), "nz": np.sin(th)}
    # for subgrid stress diffusion: centroid coordinates, the vertex viscosity (Maxwell
    # times eta/G from 1e-2 to 1e2 of dt = 1e11 s) and the shear modulus of the 3 phases
    a["xc_coord"], a["zc_coord"] = running(xmin + dx / 2.0, dx, ncx), running(zmin + dz / 2.0, dz, ncz)
    rng2 = np.random.default_rng(seed + 7)
    a["eta_phys_s"] = 10.0 ** rng2.uniform(19.0, 23.0, nv) / sc.eta
    G = np.array([3e10, 2.5e10, 4e10]) / sc.S
    model = make_model(ncx, ncz, 3, sc=sc)  # marker phases 0..2
    model.periodic_x = periodic
    return Workload("markers", model, None, a,
                    info=dict(seed=seed, ncx=ncx, ncz=ncz, dx=dx, dz=dz, markers=mk, G=G))
