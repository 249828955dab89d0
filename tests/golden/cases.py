"""Parity cases shared by the golden-fixture generator and the tests.

GRID_CASES are small grids of the benchmark workloads (all field layouts,
averaging modes, scalings, air cells, periodicity); OPERATOR_CASES run
RheologicalOperators on what a grid case's sweep produced; STRAIN_CASES run
StrainRateComponents on velocity fields (air, periodicity, one cell, ragged);
SOFTENING_CASES and SHEAR_CASES the sweep's input preparation; MARKER_CASES the
markers' stress update (UpdateParticleStress).  POINT_CASES drive
ViscosityConcise / ViscosityConciseAniso directly on random points and cover
the branches the grid workloads do not reach: Popov et al. 2025 plasticity
(plast=2, with and without the tensile line search), paleowattmeter grain size
(gs=1), constant and mixed viscosity, grain-boundary sliding, density models,
the initial step (step=0), no elasticity, and visco-plastic regularisation.
Every case is deterministic in its seed.
"""
import numpy as np

import mdz_rheo as R
import mdz_workloads as W


def _air(w):
    nx = w.model.Nx
    ncx = nx - 1
    w.arrays["BCp_type"][-3 * ncx:] = 30
    w.arrays["BCp_type"][-4 * ncx:-3 * ncx] = 31
    w.arrays["BCg_type"][-5 * nx:] = 30
    return w


def _periodic(w):
    w.model.periodic_x = 1
    return w


GRID_CASES = {
    # name: (builder, aniso, final_update)
    "plain_small": (lambda: W.plain_small(seed=0, ncx=12, ncz=10), False, 0),
    "plain_large": (lambda: W.plain_large(seed=1, ncx=12, ncz=10), False, 0),
    "plain_large_typical": (lambda: W.plain_large(seed=2, ncx=12, ncz=10, sc=W.TYPICAL), False, 0),
    "plain_large_harmonic": (lambda: W.plain_large(seed=3, ncx=11, ncz=13, eta_average=1), False, 0),
    "plain_large_geometric_periodic": (lambda: _periodic(W.plain_large(seed=4, ncx=10, ncz=12, eta_average=2)),
                                       False, 1),
    "plain_large_air": (lambda: _air(W.plain_large(seed=5, ncx=12, ncz=12)), False, 0),
    "aniso": (lambda: W.aniso(seed=6, ncx=12, ncz=10), True, 0),
    "aniso_typical_harmonic": (lambda: _set(W.aniso(seed=7, ncx=10, ncz=11, sc=W.TYPICAL), eta_average=1), True, 0),
    "plain_large_dilatant_density": (lambda: _dilatant_density(W.plain_large(seed=8, ncx=12, ncz=11)), False, 0),
}

# RheologicalOperators on the fields a grid case's sweep produced:
# name: (grid case, jacobian, compressible)
OPERATOR_CASES = {
    "plain_large_picard": ("plain_large", 0, 0),
    "plain_large_newton": ("plain_large", 1, 0),
    "plain_large_typical_newton": ("plain_large_typical", 1, 0),
    "plain_large_harmonic_newton": ("plain_large_harmonic", 1, 0),
    "plain_large_geometric_periodic_newton": ("plain_large_geometric_periodic", 1, 0),
    "plain_large_air_newton": ("plain_large_air", 1, 0),
    "dilatant_density_newton_compressible": ("plain_large_dilatant_density", 1, 1),
    "aniso_picard": ("aniso", 0, 0),
    "aniso_newton_compressible": ("aniso", 1, 1),
    "aniso_typical_harmonic_newton": ("aniso_typical_harmonic", 1, 0),
}


# StrainRateComponents on velocity fields:
# name: (builder, out_of_plane, compressible)
STRAIN_CASES = {
    "basic": (lambda: W.velocity_field(seed=11, ncx=12, ncz=10), 0, 0.0),
    "air_compressible_oop": (lambda: W.velocity_field(seed=12, ncx=13, ncz=12, air=0.3), 1, 1.0),
    "periodic_air": (lambda: W.velocity_field(seed=13, ncx=11, ncz=14, air=0.25, periodic=1), 0, 1.0),
    "one_cell": (lambda: W.velocity_field(seed=14, ncx=1, ncz=1), 1, 1.0),
    "ragged_periodic": (lambda: W.velocity_field(seed=15, ncx=45, ncz=3, air=0.4, periodic=1), 1, 0.0),
}

# CohesionFrictionDilationGrid with markers (the reference's own marker-to-grid
# interpolation runs when the fixture is made; the fixture keeps the plastic strain it
# put on the grid as the GPU path's input):
# name: (builder, smooth_softening, hardening_modulus, marker_noise, interp_stencil)
SOFTENING_CASES = {
    "piecewise": (lambda: W.prep_workload(seed=21, ncx=14, ncz=11, nphases=4, markers_per_cell=6), 0, 0, 0, 1),
    "piecewise_air_periodic_noise": (lambda: W.prep_workload(seed=22, ncx=13, ncz=12, nphases=5, air=0.3,
                                                            periodic=1, markers_per_cell=6), 0, 0, 1, 1),
    "erfc": (lambda: W.prep_workload(seed=23, ncx=12, ncz=12, nphases=3, air=0.2, markers_per_cell=6), 1, 0, 1, 1),
    "hardening_stencil9": (lambda: W.prep_workload(seed=24, ncx=15, ncz=10, nphases=4, air=0.2,
                                                  markers_per_cell=6), 0, 1, 0, 9),
}

# ShearModCompExpGrid: name: builder
SHEAR_CASES = {
    "basic": lambda: W.prep_workload(seed=31, ncx=12, ncz=10, nphases=5),
    "air_periodic": lambda: W.prep_workload(seed=32, ncx=13, ncz=11, nphases=4, air=0.3, periodic=1),
    "one_phase_typical": lambda: W.prep_workload(seed=33, ncx=9, ncz=14, nphases=1, sc=W.TYPICAL),
}

# UpdateParticleStress: name: (builder, elastic, stress_rotation, anisotropy, advection, interp_stencil)
MARKER_CASES = {
    "jaumann": (lambda: W.marker_workload(seed=41, ncx=14, ncz=11, markers_per_cell=4), 1, 1, 0, 1, 1),
    "analytical_director_air_periodic": (lambda: W.marker_workload(seed=42, ncx=13, ncz=12, markers_per_cell=5,
                                                                   air=0.3, periodic=1), 1, 2, 1, 1, 1),
    "stencil9_director_air": (lambda: W.marker_workload(seed=43, ncx=12, ncz=14, markers_per_cell=6, air=0.2),
                              1, 1, 1, 1, 9),
    "no_rotation_periodic_stencil9": (lambda: W.marker_workload(seed=44, ncx=15, ncz=10, markers_per_cell=4,
                                                                periodic=1), 1, 0, 0, 1, 9),
    "director_only": (lambda: W.marker_workload(seed=45, ncx=11, ncz=13, markers_per_cell=4, air=0.25),
                      0, 1, 1, 1, 1),
    # (builder, elastic, rotation, anisotropy, advection, stencil, subgrid_diffusion)
    "subgrid2_jaumann": (lambda: W.marker_workload(seed=46, ncx=14, ncz=12, markers_per_cell=4), 1, 1, 0, 1, 1, 2),
    "subgrid2_stencil9_director_air_periodic": (lambda: W.marker_workload(seed=47, ncx=13, ncz=11, markers_per_cell=6,
                                                                          air=0.25, periodic=1), 1, 2, 1, 1, 9, 2),
}

def _dilatant_density(w):
    """Dilation 10 deg, a finite bulk modulus and a pressure-dependent density, so the
    plastic-divergence and density derivatives of the Newton operator are exercised."""
    for k in ("dil_n", "dil_s"):
        w.arrays[k][:] = 10.0 * W.DEG
    for k in ("bet_n", "bet_s"):
        w.arrays[k][:] = 1e-11
    for p in range(w.mat.Nb_phases):
        w.mat.density_model[p] = 1
        w.mat.rho[p], w.mat.alp[p], w.mat.bet[p] = 3300.0, 3e-5, 1e-11
    return w


def _set(w, **kv):
    for k, v in kv.items():
        setattr(w.model, k, v)
    return w


# ---------------------------------------------------------------------------------------
# point cases
# ---------------------------------------------------------------------------------------
def _points(rng, n, nphases, T=(600.0, 1300.0), E=(1e-15, 1e-13), P=(0.0, 3e9), d=(1e-4, 5e-3),
            stress=5e7, aniso=False):
    pin = {}
    pin["phase"] = rng.integers(0, nphases, n).astype(np.int32)
    pin["G"] = np.full(n, 3e10)
    pin["T"] = rng.uniform(*T, n)
    pin["P"] = rng.uniform(*P, n)
    pin["d"] = W.loguniform(rng, d[0], d[1], n)
    pin["phi"] = np.zeros(n)
    pin["X0"] = np.zeros(n)
    exx = W.signed_loguniform(rng, E[0], E[1], n)
    pin["Exx"], pin["Ezz"] = exx, -exx
    pin["Exz"] = W.signed_loguniform(rng, E[0], E[1], n)
    t0 = rng.uniform(-stress, stress, n)
    pin["Txx0"], pin["Tzz0"] = t0, -t0
    pin["Txz0"] = rng.uniform(-stress, stress, n)
    pin["strain_acc"] = np.zeros(n)
    pin["dil"] = np.zeros(n)
    pin["fric"] = np.full(n, 30.0 * W.DEG)
    pin["C"] = np.full(n, 1e7)
    pin["P0"] = pin["P"].copy()
    pin["T0"] = pin["T"].copy()
    pin["beta"] = np.full(n, 1e-40)
    pin["div"] = np.zeros(n)
    if aniso:
        th = rng.uniform(0, np.pi, n)
        lay = th - np.pi / 2
        pin["lxlz"], pin["lx2"] = np.cos(lay) * np.sin(lay), np.cos(lay) ** 2
        pin["angle"], pin["ani_fac"] = th, W.loguniform(rng, 1.0, 10.0, n)
    return pin


def _popov(ls):
    def build(seed):
        rng = np.random.default_rng(seed)
        m = W.empty_materials(2)
        W.set_power_law(m, 0, **W.OLIVINE_DRY)
        W.set_power_law(m, 1, **W.SOFT_QTZ)
        for p in range(2):
            m.plast[p] = 2
            m.T_st[p] = -5e6
        md = W.make_model(8, 8, 2)
        md.tensile_line_search = ls
        pin = _points(rng, 200, 2, P=(-2e7, 2e8), stress=1e8, E=(1e-14, 1e-12))
        pin["dil"] = np.full(200, 5.0 * W.DEG)
        pin["beta"] = np.full(200, 1e-11)
        return md, m, pin
    return build


def _gse(aniso):
    def build(seed):
        rng = np.random.default_rng(seed)
        m = W.empty_materials(2)
        W.set_power_law(m, 0, **W.OLIVINE_DRY)
        W.set_linear(m, 0, **W.OLIVINE_DIFF)
        W.set_power_law(m, 1, **W.OLIVINE_DRY)
        for p in range(2):
            m.gs[p] = 1
            m.Kpzm[p], m.Qpzm[p], m.Gpzm[p], m.Lpzm[p], m.cpzm[p], m.ppzm[p] = 1.5e-5, 2.0e5, 1.0, 0.1, np.pi, 3.0
        md = W.make_model(8, 8, 2)
        pin = _points(rng, 120, 2, T=(900.0, 1400.0), E=(1e-15, 1e-13), aniso=aniso)
        return md, m, pin
    return build


def _constant_mix(seed):
    rng = np.random.default_rng(seed)
    m = W.empty_materials(3)
    m.cstv[0] = 1
    m.eta0[0] = 1e21
    m.cstv[1] = 1
    m.eta0[1] = 5e19
    W.set_power_law(m, 1, **W.SOFT_QTZ)
    m.cstv[2] = 1
    m.eta0[2] = 3e22
    m.phase_mix[2] = 1
    m.phase_two[2] = 0
    m.gbsv[1] = 1
    m.Qgbs[1], m.Vgbs[1], m.ngbs[1], m.mgbs[1], m.Agbs[1], m.Fgbs[1] = 400e3, 0.0, 3.5, 2.0, 6.5e-40, 1.0
    md = W.make_model(8, 8, 3)
    md.diffuse_X = 1
    md.diffuse_avg = seed % 3
    pin = _points(rng, 150, 3)
    pin["X0"] = rng.uniform(0.0, 1.0, 150)
    return md, m, pin


def _density(seed):
    rng = np.random.default_rng(seed)
    m = W.materials_plain_large(4)
    for p, dm in enumerate((0, 1, 3, 5)):
        m.density_model[p] = dm
        m.rho[p] = 3000.0 + 100 * p
        m.alp[p] = 3e-5
        m.bet[p] = 1e-11
        m.drho[p] = -300.0
    md = W.make_model(8, 8, 4)
    md.density_variations = 1
    pin = _points(rng, 160, 4)
    pin["phi"] = rng.uniform(0.0, 0.1, 160)
    return md, m, pin


def _step0(seed):
    rng = np.random.default_rng(seed)
    m = W.materials_plain_large(5)
    md = W.make_model(8, 8, 5)
    md.step = 0
    return md, m, _points(rng, 150, 5)


def _no_elastic(seed):
    # Without elasticity nothing bounds the trial stress; below ~1100 K the cold
    # diffusion-only phase reaches Tii > 1e4 Tyield, where the reference's return
    # Tiic = Tii - eta gdot is cancellation noise.  Keep T where it is well conditioned.
    rng = np.random.default_rng(seed)
    m = W.materials_plain_large(5)
    md = W.make_model(8, 8, 5)
    md.elastic = 0
    return md, m, _points(rng, 150, 5, T=(1100.0, 1500.0))


def _viscoplastic(seed):
    rng = np.random.default_rng(seed)
    m = W.materials_plain_small()
    for p in range(2):
        m.eta_vp[p] = 1e20
        m.Slim[p] = 5e8
    md = W.make_model(8, 8, 2)
    pin = _points(rng, 150, 2, E=(1e-14, 1e-12), stress=2e8)
    pin["dil"] = np.full(150, 2.0 * W.DEG)
    pin["beta"] = np.full(150, 1e-11)
    return md, m, pin


def _large_mix(aniso):
    def build(seed):
        rng = np.random.default_rng(seed)
        m = W.materials_plain_large(5)
        if aniso:
            for p in range(5):
                m.gs[p] = 0
        md = W.make_model(8, 8, 5)
        return md, m, _points(rng, 250, 5, T=(400.0, 1550.0), aniso=aniso)
    return build


POINT_CASES = {
    # name: (builder(seed), aniso, centroid, final_update)
    "popov": (_popov(0), False, 1, 0),
    "popov_line_search": (_popov(1), False, 1, 1),
    "gse": (_gse(False), False, 1, 0),
    "gse_aniso": (_gse(True), True, 1, 0),
    "constant_mix_gbs": (_constant_mix, False, 1, 0),
    "density_models": (_density, False, 1, 1),
    "step0": (_step0, False, 1, 0),
    "no_elastic": (_no_elastic, False, 0, 0),
    "viscoplastic": (_viscoplastic, False, 1, 0),
    "large_mix_peierls_cutoff": (_large_mix(False), False, 1, 0),
    "aniso_mix": (_large_mix(True), True, 1, 0),
}


def point_case(name, seed=0):
    build, aniso, centroid, fu = POINT_CASES[name]
    md, m, pin = build(seed)
    return md, m, pin, aniso, centroid, fu


def alloc_point_outputs(n):
    out = {k: np.zeros(n) for k in R.PT_OUT}
    out["iters"] = np.zeros(n, np.int32)
    out["status"] = np.zeros(n, np.int32)
    return out
