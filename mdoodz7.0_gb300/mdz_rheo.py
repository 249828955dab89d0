"""Python binding of the GB300 local-rheology library (include/mdz_rheo.h).

This is the host-side mirror of MDOODZ7.0's interface for the local rheology
update: `sweep` plays NonNewtonianViscosityGrid (MDLIB/RheologyDensity.c:1131),
`sweep_aniso` NonNewtonianViscosityGridAniso (MDLIB/AnisotropyRoutines.c:885)
and `points` ViscosityConcise / ViscosityConciseAniso per point
(MDLIB/RheologyDensity.c:385, MDLIB/AnisotropyRoutines.c:282).  Field names
are the reference's `grid` member names (MDLIB/mdoodz-private.h:75-147).

Everything goes through the C ABI with ctypes; buffers are numpy arrays
(host memory) or torch CUDA tensors (device memory).  There is no CPU
fallback: if the CUDA library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libmdz_rheo_gb300.so")

MAX_PHASES = 20

# ---- status codes (include/mdz_rheo.h) ----------------------------------
MDZ_OK = 0
MDZ_EINVAL = -1
MDZ_ECUDA = -2
MDZ_EUNSUPPORTED = -3
MDZ_ENOMEM = -4
MDZ_ENOTREADY = -5
MDZ_EVE_ITER = -10
MDZ_EGSE_ITER = -11
MDZ_ESINGULAR = -12
MDZ_EEMPTY_CELL = -13
MDZ_ENONFINITE = -14
MDZ_EWDISS = -15
MDZ_EGRAIN_ZERO = -16
MDZ_ELINESEARCH = -17
MDZ_EANISO_NAN = -18
MDZ_EANISO_ITER = -19
MDZ_ESCRATCH = -20
MDZ_ESHEAR_INF = -21
MDZ_EMARKER_OUT = -22
STATIC_SCRATCH_BYTES = 4 << 20

MEM_HOST = 0
MEM_DEVICE = 1
SWEEP_ASYNC = 0x1
SWEEP_WARMSTART = 0x2
SWEEP_ITERS = 0x4
SWEEP_REF_START = 0x8
SWEEP_WARM_TILES = 0x10
SWEEP_STAGED = 0x20  # host memory: stage through device copies even where the GPU can address the arrays
OPS_PER_NODE = 0x40  # operators: the isotropic Newton operator one thread per node (same bits)
# per-(node, phase) item words of SWEEP_ITERS: iterations in bits 0-7, then mechanism bits
MECH_CONSTANT, MECH_DISLOCATION, MECH_PEIERLS, MECH_DIFFUSION = 1 << 8, 1 << 9, 1 << 10, 1 << 11
MECH_GBS, MECH_GRAIN_SIZE, MECH_PLASTIC, MECH_ELASTIC, MECH_YIELD = 1 << 12, 1 << 13, 1 << 14, 1 << 15, 1 << 16
DEFAULT_POLISH = 4
START_DD = 0x100
DEFAULT_START = DEFAULT_POLISH | START_DD

# ---- struct layouts (must follow include/mdz_rheo.h field by field) -------
MAT_INT = ["cstv", "pwlv", "linv", "gbsv", "expv", "gs", "kin", "plast", "density_model",
           "phase_mix", "phase_two", "reac_soft", "reac_phase", "melt"]
MAT_DBL = ["eta0", "rho", "drho", "alp", "bet", "T0", "P0", "Slim", "eta_vp", "n_vp", "T_st", "gs_ref",
           "Qpwl", "Vpwl", "npwl", "mpwl", "rpwl", "Apwl", "fpwl", "apwl", "Fpwl", "pref_pwl",
           "Qlin", "Vlin", "nlin", "mlin", "rlin", "Alin", "flin", "alin", "Flin",
           "Qgbs", "Vgbs", "ngbs", "mgbs", "rgbs", "Agbs", "fgbs", "agbs", "Fgbs",
           "Qexp", "Sexp", "Eexp", "Gexp", "nexp",
           "Kpzm", "Qpzm", "Gpzm", "Lpzm", "cpzm", "ppzm"]


class Materials(C.Structure):
    _fields_ = ([("Nb_phases", C.c_int), ("R", C.c_double)]
                + [(n, C.c_int * MAX_PHASES) for n in MAT_INT]
                + [(n, C.c_double * MAX_PHASES) for n in MAT_DBL])


MODEL_INT = ["Nx", "Nz", "Nb_phases", "step", "elastic", "eta_average", "periodic_x",
             "density_variations", "tensile_line_search", "melting", "chemical_production",
             "diffuse_X", "diffuse_avg"]
MODEL_DBL = ["dt", "min_eta", "max_eta", "eta_tol", "scale_eta", "scale_L", "scale_T", "scale_S",
             "scale_E"]


class Model(C.Structure):
    _fields_ = [(n, C.c_int) for n in MODEL_INT] + [(n, C.c_double) for n in MODEL_DBL]


CEN_IN = ["mu_n", "T", "p_in", "d0_n", "phi0_n", "X0_n", "exxd", "ezzd", "exz_n", "sxxd0", "szzd0",
          "sxz0_n", "strain_n", "dil_n", "fric_n", "C_n", "p0_n", "T0_n", "bet_n", "div_u"]
VER_IN = ["mu_s", "X0_s", "exxd_s", "ezzd_s", "exz", "sxxd0_s", "szzd0_s", "sxz0", "strain_s",
          "dil_s", "fric_s", "C_s", "p0_s", "bet_s", "div_u_s"]
ANI_IN_N = ["d1_n", "d2_n", "angle_n", "aniso_factor_n"]
ANI_IN_S = ["d1_s", "d2_s", "angle_s", "aniso_factor_s"]
VER_INTERP = ["T_s", "P_s", "d0_s", "phi0_s"]
CEN_OUT = ["eta_n", "eta_phys_n", "VE_n", "sxxd", "szzd", "sxz_n", "eII_el", "eII_pl", "eII_pwl",
           "eII_exp", "eII_lin", "eII_gbs", "eII_cst", "d_n", "p_corr", "div_u_el", "div_u_pl",
           "div_u_r", "Wtot", "Wel", "Wdiss", "X_n", "OverS_n", "rho_n"]
VER_OUT = ["sxxd_s", "szzd_s", "sxz", "eta_phys_s", "eta_s", "X_s", "VE_s"]

_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)


class GridFields(C.Structure):
    _fields_ = ([(n, _P) for n in CEN_IN] + [("phase_perc_n", _PP), ("BCp_type", _P)]
                + [(n, _P) for n in VER_IN] + [("phase_perc_s", _PP), ("BCg_type", _P)]
                + [(n, _P) for n in ANI_IN_N + ANI_IN_S] + [(n, _P) for n in VER_INTERP]
                + [(n, _P) for n in CEN_OUT] + [("phase_eta_n", _PP)]
                + [(n, _P) for n in VER_OUT] + [("phase_eta_s", _PP)])


class SweepStats(C.Structure):
    _fields_ = [("phase_calls", C.c_uint64), ("newton_iters", C.c_uint64),
                ("max_newton_iters", C.c_uint32), ("plastic_calls", C.c_uint64),
                ("status", C.c_int32), ("error_node", C.c_int64), ("elapsed_ms", C.c_double),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("kernel_launches", C.c_uint32),
                ("mma_fault", C.c_uint32), ("fp32_steps", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


OPS_N = ["D11_n", "D12_n", "D13_n", "D14_n", "D21_n", "D22_n", "D23_n", "D24_n", "drhodp_n"]
OPS_S = ["D31_s", "D32_s", "D33_s", "D34_s"]


class OperatorFields(C.Structure):
    """mdz_operator_fields: the D coefficients of RheologicalOperators."""
    _fields_ = [(n, _P) for n in OPS_N + OPS_S]


def make_operator_fields(arrays: Dict[str, object]) -> OperatorFields:
    o = OperatorFields()
    for name in OPS_N + OPS_S:
        setattr(o, name, _ptr(arrays.get(name)))
    return o


def alloc_operator_fields(nc: int, nv: int, like=None) -> Dict[str, object]:
    """Zeroed D arrays (numpy, or torch on the device of `like`)."""
    if like is not None:
        import torch
        return {**{k: torch.zeros(nc, dtype=torch.float64, device=like.device) for k in OPS_N},
                **{k: torch.zeros(nv, dtype=torch.float64, device=like.device) for k in OPS_S}}
    return {**{k: np.zeros(nc) for k in OPS_N}, **{k: np.zeros(nv) for k in OPS_S}}


SR_N = ["div_u", "exxd", "ezzd", "exz_n", "wxz_n"]
SR_S = ["exz", "wxz", "exxd_s", "ezzd_s", "div_u_s"]


class StrainRateFields(C.Structure):
    """mdz_strain_rate_fields: velocities in, strain rates and spin out (StrainRateComponents)."""
    _fields_ = [("u_in", _P), ("v_in", _P), ("BCp_type", _P), ("BCg_type", _P)] + [(n, _P) for n in SR_N + SR_S]


def make_strain_rate_fields(arrays: Dict[str, object]) -> StrainRateFields:
    o = StrainRateFields()
    for name, _ in StrainRateFields._fields_:
        setattr(o, name, _ptr(arrays.get(name)))
    return o


def alloc_strain_rate_fields(nc: int, nv: int, like=None) -> Dict[str, object]:
    """Zeroed output arrays of StrainRateComponents (numpy, or torch on the device of `like`)."""
    if like is not None:
        import torch
        return {**{k: torch.zeros(nc, dtype=torch.float64, device=like.device) for k in SR_N},
                **{k: torch.zeros(nv, dtype=torch.float64, device=like.device) for k in SR_S}}
    return {**{k: np.zeros(nc) for k in SR_N}, **{k: np.zeros(nv) for k in SR_S}}


MLP_IN, MLP_HID = 16, 64


class MlpWeights(C.Structure):
    """mdz_mlp_weights: the warm-start perceptron (row-major [out][in] FP32 weights)."""
    _fields_ = [("n_feat", C.c_int32),
                ("W1", C.c_float * (MLP_HID * MLP_IN)), ("b1", C.c_float * MLP_HID),
                ("W2", C.c_float * (MLP_HID * MLP_HID)), ("b2", C.c_float * MLP_HID),
                ("W3", C.c_float * (2 * MLP_HID)), ("b3", C.c_float * 2),
                ("x_shift", C.c_float * MLP_IN), ("x_scale", C.c_float * MLP_IN),
                ("z_shift", C.c_float), ("z_scale", C.c_float)]

    def arrays(self):
        return {"W1": np.ctypeslib.as_array(self.W1).reshape(MLP_HID, MLP_IN),
                "b1": np.ctypeslib.as_array(self.b1),
                "W2": np.ctypeslib.as_array(self.W2).reshape(MLP_HID, MLP_HID),
                "b2": np.ctypeslib.as_array(self.b2),
                "W3": np.ctypeslib.as_array(self.W3).reshape(2, MLP_HID),
                "b3": np.ctypeslib.as_array(self.b3),
                "x_shift": np.ctypeslib.as_array(self.x_shift), "x_scale": np.ctypeslib.as_array(self.x_scale)}

    def save(self, path):
        np.savez(path, raw=np.frombuffer(bytes(self), dtype=np.uint8))

    @classmethod
    def load(cls, path):
        raw = np.load(path)["raw"]
        w = cls()
        C.memmove(C.addressof(w), raw.tobytes(), C.sizeof(w))
        return w


class MlpTrainCfg(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("lr_final", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float), ("w_pl", C.c_float),
                ("seed", C.c_uint64)]


PT_IN = ["G", "T", "P", "d", "phi", "X0", "Exx", "Ezz", "Exz", "Txx0", "Tzz0", "Txz0", "strain_acc",
         "dil", "fric", "C", "P0", "T0", "beta", "div"]
PT_ANI = ["lxlz", "lx2", "angle", "ani_fac"]
PT_OUT = ["eta", "Txx", "Tzz", "Txz", "etaVE", "VEcoeff", "Eii_el", "Eii_pl", "Eii_pwl", "Eii_exp",
          "Eii_lin", "Eii_gbs", "Eii_cst", "d1", "X1", "OverS", "Pcorr", "rho", "div_el", "div_pl",
          "div_r", "Wtot", "Wel", "Wdiss"]


class PointInputs(C.Structure):
    _fields_ = ([("phase", _P)] + [(n, _P) for n in PT_IN] + [(n, _P) for n in PT_ANI]
                + [("post_process", C.c_int), ("centroid", C.c_int), ("final_update", C.c_int)])


class PointOutputs(C.Structure):
    _fields_ = [(n, _P) for n in PT_OUT] + [("iters", _P), ("status", _P)]


# ---- buffer helpers ---------------------------------------------------------
def _ptr(a) -> Optional[int]:
    """Address of a numpy array or torch tensor (None stays NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"], "arrays must be contiguous"
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _ptr_array(lst):
    if lst is None:
        return None
    arr = (C.c_void_p * max(1, len(lst)))(*[_ptr(a) for a in lst])
    return arr


class FieldSet:
    """A dict of grid arrays plus the mdz_grid_fields struct that points at them.

    `arrays` maps reference field names to arrays; `phase_perc_n`,
    `phase_perc_s`, `phase_eta_n`, `phase_eta_s` map to lists (one array per
    phase).  Missing names become NULL.
    """

    def __init__(self, arrays: Dict[str, object]):
        self.arrays = arrays
        self._keep = []
        s = GridFields()
        for name, _ in GridFields._fields_:
            v = arrays.get(name)
            if name.startswith("phase_"):
                pa = _ptr_array(v)
                self._keep.append(pa)
                setattr(s, name, C.cast(pa, _PP) if pa is not None else None)
            else:
                setattr(s, name, _ptr(v))
        self.struct = s

    def __getitem__(self, k):
        return self.arrays[k]


PREP_MAT_DBL = ["G", "bet", "alp", "C", "phi", "psi", "H_c", "C_end", "phi_end", "psi_end", "pls_start", "pls_end"]
PREP_MAT_INT = ["phi_soft", "psi_soft", "coh_soft"]
SOFT_N, SOFT_S = ["fric_n", "dil_n", "C_n"], ["fric_s", "dil_s", "C_s"]
MOD_N, MOD_S = ["mu_n", "bet_n", "alp"], ["mu_s", "bet_s"]


class PrepMaterials(C.Structure):
    """mdz_prep_materials: the mat_prop fields of Softening and ShearModCompExpGrid."""
    _fields_ = ([("Nb_phases", C.c_int)] + [(n, C.c_double * MAX_PHASES) for n in PREP_MAT_DBL]
                + [(n, C.c_int * MAX_PHASES) for n in PREP_MAT_INT])


class PrepFields(C.Structure):
    """mdz_prep_fields: grid arrays of the preparation steps."""
    _fields_ = ([("phase_perc_n", _PP), ("phase_perc_s", _PP), ("BCp_type", _P), ("BCg_type", _P),
                 ("strain_pl_n", _P), ("strain_pl_s", _P), ("noise_n", _P), ("noise_s", _P)]
                + [(n, _P) for n in SOFT_N + SOFT_S + MOD_N + MOD_S])


class PrepFieldSet:
    """A dict of preparation arrays (phase_perc_n/_s are lists) and the struct over it."""

    def __init__(self, arrays: Dict[str, object]):
        self.arrays = arrays
        s = PrepFields()
        self._keep = []
        for name, _ in PrepFields._fields_:
            v = arrays.get(name)
            if name.startswith("phase_"):
                pa = _ptr_array(v)
                self._keep.append(pa)
                setattr(s, name, C.cast(pa, _PP) if pa is not None else None)
            else:
                setattr(s, name, _ptr(v))
        self.struct = s


class Markers(C.Structure):
    """mdz_markers: the marker arrays of UpdateParticleStress."""
    _fields_ = [("n", C.c_int64), ("x", _P), ("z", _P), ("phase", _P), ("sxxd", _P), ("szzd", _P), ("sxz", _P),
                ("nx", _P), ("nz", _P)]


MARKER_GRID_IN = ["xg_coord", "zg_coord", "xvz_coord", "zvx_coord", "BCp_type", "BCg_type", "sxxd", "szzd", "sxxd0",
                  "szzd0", "sxz", "sxz0", "u_in", "v_in", "wxz", "xc_coord", "zc_coord", "eta_phys_s"]
MARKER_ARRAYS = ["x", "z", "phase", "sxxd", "szzd", "sxz", "nx", "nz"]


class MarkerGrid(C.Structure):
    """mdz_marker_grid: the grid side of UpdateParticleStress."""
    _fields_ = [("dx", C.c_double), ("dz", C.c_double)] + [(n, _P) for n in MARKER_GRID_IN]


class MarkerOpts(C.Structure):
    """mdz_marker_opts: the params switches of UpdateParticleStress and, for subgrid
    diffusion 2, the per-phase shear modulus (`set_G` keeps the array alive)."""
    _fields_ = [(n, C.c_int) for n in ("elastic", "subgrid_diffusion", "stress_rotation", "anisotropy", "advection",
                                        "interp_stencil")] + [("G", _P)]

    def set_G(self, G):
        self._G = np.ascontiguousarray(G, np.float64)
        self.G = self._G.ctypes.data
        return self


def make_marker_structs(grid: Dict[str, object], markers: Dict[str, object], dx: float, dz: float):
    g = MarkerGrid()
    g.dx, g.dz = dx, dz
    for n in MARKER_GRID_IN:
        setattr(g, n, _ptr(grid.get(n)))
    m = Markers()
    x = markers["x"]
    m.n = int(x.numel() if hasattr(x, "numel") else x.size)
    for n in MARKER_ARRAYS:
        setattr(m, n, _ptr(markers.get(n)))
    return g, m


def make_points(inputs: Dict[str, object], outputs: Dict[str, object], post_process=1, centroid=1,
                final_update=0):
    pi = PointInputs()
    for name, _ in PointInputs._fields_:
        if name in ("post_process", "centroid", "final_update"):
            continue
        setattr(pi, name, _ptr(inputs.get(name)))
    pi.post_process, pi.centroid, pi.final_update = post_process, centroid, final_update
    po = PointOutputs()
    for name, _ in PointOutputs._fields_:
        setattr(po, name, _ptr(outputs.get(name)))
    return pi, po


# ---- library ----------------------------------------------------------------
class RheoError(RuntimeError):
    def __init__(self, code, where=""):
        self.code = code
        super().__init__(f"{where}: {status_string(code)} ({code})")


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libmdz_rheo_gb300.so.  Raises if it was not built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"GB300 rheology library not built: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    lib.mdz_rheo_version.restype = C.c_int
    lib.mdz_rheo_status_string.restype = C.c_char_p
    lib.mdz_rheo_status_string.argtypes = [C.c_int]
    lib.mdz_rheo_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    lib.mdz_rheo_destroy.argtypes = [C.c_void_p]
    lib.mdz_rheo_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    lib.mdz_rheo_set_host_bands.argtypes = [C.c_void_p, C.c_int]
    lib.mdz_rheo_host_access.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    lib.mdz_rheo_sync.argtypes = [C.c_void_p, C.POINTER(SweepStats)]
    for fn in (lib.mdz_rheo_sweep, lib.mdz_rheo_sweep_aniso):
        fn.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(Materials), C.POINTER(GridFields),
                       C.c_int, C.c_int, C.c_int, C.POINTER(SweepStats)]
    lib.mdz_rheo_points.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(Materials),
                                    C.POINTER(PointInputs), C.POINTER(PointOutputs), C.c_int64,
                                    C.c_int, C.c_int]
    lib.mdz_rheo_get_iterations.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.mdz_rheo_abi_sizes.argtypes = [C.POINTER(C.c_size_t)]
    lib.mdz_rheo_measure_fp64_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    lib.mdz_rheo_math_selftest.argtypes = [C.c_int, C.c_void_p, C.c_int64] + [C.c_void_p] * 4
    lib.mdz_rheo_div_selftest.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p]
    lib.mdz_rheo_ceil_selftest.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    lib.mdz_rheo_dd_selftest.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_void_p]
    lib.mdz_rheo_quotient_selftest.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    lib.mdz_rheo_points_static.argtypes = [C.POINTER(Model), C.POINTER(Materials), C.POINTER(PointInputs),
                                           C.POINTER(PointOutputs), C.c_int64, C.c_int, C.c_int, C.c_void_p,
                                           C.POINTER(SweepStats)]
    lib.mdz_rheo_batch_create.argtypes = [C.c_void_p, C.c_int, C.POINTER(Model), C.POINTER(Materials),
                                          C.POINTER(GridFields), C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_void_p)]
    lib.mdz_rheo_batch_destroy.argtypes = [C.c_void_p]
    lib.mdz_rheo_batch_sweep.argtypes = [C.c_void_p, C.POINTER(SweepStats)]
    lib.mdz_rheo_batch_capture.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_uint64]
    lib.mdz_rheo_batch_launch.argtypes = [C.c_void_p, C.POINTER(SweepStats)]
    lib.mdz_rheo_batch_set_grid.argtypes = [C.c_void_p, C.c_int]
    lib.mdz_rheo_operators.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(Materials), C.POINTER(GridFields),
                                       C.POINTER(OperatorFields), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(SweepStats)]
    lib.mdz_rheo_strain_rates.argtypes = [C.c_void_p, C.POINTER(Model), C.c_double, C.c_double, C.c_int,
                                          C.c_double, C.POINTER(StrainRateFields), C.c_int, C.c_int,
                                          C.POINTER(SweepStats)]
    lib.mdz_rheo_softening.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(PrepMaterials), C.POINTER(PrepFields),
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(SweepStats)]
    lib.mdz_rheo_shear_modulus.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(PrepMaterials),
                                           C.POINTER(PrepFields), C.c_int, C.c_int, C.POINTER(SweepStats)]
    lib.mdz_rheo_marker_stress.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(MarkerOpts), C.POINTER(MarkerGrid),
                                           C.POINTER(Markers), C.c_int, C.c_int, C.POINTER(SweepStats)]
    lib.mdz_rheo_p2mastah.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(MarkerGrid), C.POINTER(Markers),
                                      C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                      C.POINTER(SweepStats)]
    lib.mdz_rheo_autotune.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(Materials), C.POINTER(GridFields),
                                      C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int)]
    lib.mdz_rheo_get_launch_shape.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.mdz_rheo_get_launch_form.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    lib.mdz_rheo_set_launch_shape.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.mdz_rheo_set_warmstart.argtypes = [C.c_void_p, C.POINTER(MlpWeights), C.c_int]
    lib.mdz_rheo_set_mma_poll_limit.argtypes = [C.c_void_p, C.c_int32]
    lib.mdz_rheo_collect.argtypes = [C.c_void_p, C.POINTER(Model), C.POINTER(Materials), C.POINTER(GridFields),
                                     C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(SweepStats)]
    lib.mdz_rheo_train_mlp.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int,
                                       C.POINTER(MlpTrainCfg), C.POINTER(MlpWeights), C.c_void_p, C.c_int]
    lib.mdz_rheo_mlp_predict.argtypes = [C.c_void_p, C.POINTER(MlpWeights), C.c_void_p, C.c_void_p, C.c_int64,
                                         C.c_int]
    lib.mdz_rheo_mlp_gradient.argtypes = [C.c_void_p, C.POINTER(MlpWeights), C.c_void_p, C.c_void_p,
                                          C.c_int64, C.c_float, C.POINTER(MlpWeights), C.c_void_p, C.c_int]
    _lib = lib
    return lib


def status_string(code: int) -> str:
    try:
        return load_library().mdz_rheo_status_string(code).decode()
    except Exception:  # library absent: still give a readable message
        return f"status {code}"


def abi_sizes():
    """sizeof() of the C structs as compiled into the library, for ABI checks."""
    lib = load_library()
    out = (C.c_size_t * 8)()
    lib.mdz_rheo_abi_sizes(out)
    return list(out)


def measure_fp64_peak(device: int = 0) -> float:
    """Measured DFMA throughput of the GPU in TFLOP/s (mdz_rheo_measure_fp64_peak)."""
    v = C.c_double()
    rc = load_library().mdz_rheo_measure_fp64_peak(device, C.byref(v))
    if rc != MDZ_OK:
        raise RheoError(rc, "mdz_rheo_measure_fp64_peak")
    return v.value


def points_static(model, mat, pin, pout, n, aniso=0, mem=MEM_HOST, stream=None, lib=None):
    """mdz_rheo_points_static: the point path on the current device, allocating nothing.
    Returns (status, SweepStats)."""
    lib = lib or load_library()
    st = SweepStats()
    rc = lib.mdz_rheo_points_static(C.byref(model), C.byref(mat), C.byref(pin), C.byref(pout), n, aniso, mem,
                                    stream, C.byref(st))
    return rc, st


def math_selftest(x: np.ndarray, device: int = 0):
    """(fast_exp, cuda_exp, fast_log, cuda_log) of the float64 array x on the GPU."""
    x = np.ascontiguousarray(x, np.float64)
    outs = [np.empty_like(x) for _ in range(4)]
    rc = load_library().mdz_rheo_math_selftest(device, x.ctypes.data, x.size, *[o.ctypes.data for o in outs])
    if rc != MDZ_OK:
        raise RheoError(rc, "mdz_rheo_math_selftest")
    return outs


def div_selftest(a: np.ndarray, b: float, device: int = 0):
    """(known-divisor division, CUDA's division) of the float64 array a by b on the GPU."""
    a = np.ascontiguousarray(a, np.float64)
    fast, plain = np.empty_like(a), np.empty_like(a)
    rc = load_library().mdz_rheo_div_selftest(device, a.ctypes.data, a.size, b, fast.ctypes.data, plain.ctypes.data)
    if rc != MDZ_OK:
        raise RheoError(rc, "mdz_rheo_div_selftest")
    return fast, plain


def quotient_selftest(r: np.ndarray, den: np.ndarray, device: int = 0):
    """r / den by the local solve's output quotient (two Newton steps on the reciprocal
    estimate) on the GPU, for float64 arrays of one shape."""
    r = np.ascontiguousarray(r, np.float64)
    den = np.ascontiguousarray(den, np.float64)
    assert r.shape == den.shape
    out = np.empty_like(r)
    rc = load_library().mdz_rheo_quotient_selftest(device, r.ctypes.data, den.ctypes.data, r.size, out.ctypes.data)
    if rc != MDZ_OK:
        raise RheoError(rc, "mdz_rheo_quotient_selftest")
    return out


def ceil_selftest(q: np.ndarray, device: int = 0):
    """(integer-pipe ceil as int32, CUDA's ceil) of the float64 array q on the GPU."""
    q = np.ascontiguousarray(q, np.float64)
    fast, plain = np.empty(q.size, np.int32), np.empty_like(q)
    rc = load_library().mdz_rheo_ceil_selftest(device, q.ctypes.data, q.size, fast.ctypes.data, plain.ctypes.data)
    if rc != MDZ_OK:
        raise RheoError(rc, "mdz_rheo_ceil_selftest")
    return fast, plain


def dd_selftest(x: np.ndarray, device: int = 0):
    """(x, exp(x), log(float32(x))) of the float64 array x as double-float (hi, lo) float32 pairs, each of shape
    (n, 2), from the GPU."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty((x.size, 6), np.float32)
    rc = load_library().mdz_rheo_dd_selftest(device, x.ctypes.data, x.size, out.ctypes.data)
    if rc != MDZ_OK:
        raise RheoError(rc, "mdz_rheo_dd_selftest")
    return out[:, 0:2], out[:, 2:4], out[:, 4:6]


def python_struct_sizes():
    return [C.sizeof(Materials), C.sizeof(Model), C.sizeof(GridFields), C.sizeof(SweepStats),
            C.sizeof(PointInputs), C.sizeof(PointOutputs)]


class Batch:
    """Many device-resident grids swept together, one launch per kind of node (mdz_rheo_batch_*).  `fieldsets` are
    FieldSets over device tensors; they (and their tensors) must outlive the batch."""

    def __init__(self, ctx: "Context", models, mats, fieldsets, aniso=False, final_update=0, flags=0):
        n = len(models)
        self.ctx = ctx
        self.lib = ctx.lib
        self._keep = list(fieldsets)
        self._models = (Model * n)(*models)
        self._mats = (Materials * n)(*mats)
        self._fields = (GridFields * n)(*[fs.struct for fs in fieldsets])
        h = C.c_void_p()
        rc = self.lib.mdz_rheo_batch_create(ctx.handle, n, self._models, self._mats, self._fields, int(aniso),
                                            final_update, flags, C.byref(h))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_batch_create")
        self.handle = h

    def sweep(self, check=True):
        st = SweepStats()
        rc = self.lib.mdz_rheo_batch_sweep(self.handle, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_batch_sweep")
        return rc, st

    def capture(self, nsweeps: int, amp: float = 0.0, seed: int = 0):
        rc = self.lib.mdz_rheo_batch_capture(self.handle, nsweeps, amp, seed)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_batch_capture")

    def launch(self, check=True):
        st = SweepStats()
        rc = self.lib.mdz_rheo_batch_launch(self.handle, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_batch_launch")
        return rc, st

    def set_grid(self, ctas: int):
        """0: one CTA per tile (default); ctas > 0: a persistent grid of that many CTAs
        striding over the tiles.  Drops a captured graph."""
        rc = self.lib.mdz_rheo_batch_set_grid(self.handle, int(ctas))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_batch_set_grid")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mdz_rheo_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def perturb_reference(x: np.ndarray, amp: float, seed: int, sweep: int, grid: int, comp: int,
                      node_offset: int = 0) -> np.ndarray:
    """Host statement of the batch strain-rate perturbation (mdz_rheo_batch_capture):
    x * (1 + amp u) with u from SplitMix64; node index = node_offset + position."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)

    def sm(z):
        z = (np.asarray(z, np.uint64) + np.uint64(0x9e3779b97f4a7c15)) & M
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xbf58476d1ce4e5b9)) & M
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94d049bb133111eb)) & M
        return z ^ (z >> np.uint64(31))

    with np.errstate(over="ignore"):
        key = sm(sm(np.uint64(seed) ^ np.uint64(sweep)) ^ np.uint64(grid))
        node = np.arange(x.size, dtype=np.uint64) + np.uint64(node_offset)
        h = sm(key ^ (node * np.uint64(3) + np.uint64(comp)))
    u = (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -52 - 1.0
    return x * (1.0 + amp * u)


class Context:
    """One mdz_rheo_ctx: a CUDA stream plus device mirrors for host-memory sweeps."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.mdz_rheo_create(device, C.byref(h))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_create")
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.mdz_rheo_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: Optional[int]):
        rc = self.lib.mdz_rheo_set_stream(self.handle, stream_ptr)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_set_stream")

    def pageable_in_place(self) -> bool:
        """Whether MDZ_MEM_HOST calls use ordinary pageable host arrays in place."""
        v = C.c_int()
        rc = self.lib.mdz_rheo_host_access(self.handle, C.byref(v))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_host_access")
        return bool(v.value)

    def set_host_bands(self, bands: int = 0):
        """Row bands of host-memory sweeps (0: automatic)."""
        rc = self.lib.mdz_rheo_set_host_bands(self.handle, bands)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_set_host_bands")

    def _sweep(self, fn, model, mat, fields, final_update, mem, flags, check):
        st = SweepStats()
        rc = fn(self.handle, C.byref(model), C.byref(mat), C.byref(fields.struct), final_update, mem,
                flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, fn.__name__)
        return rc, st

    def sweep(self, model, mat, fields, final_update=0, mem=MEM_HOST, flags=0, check=True):
        """NonNewtonianViscosityGrid on `fields` (a FieldSet).  Returns (status, SweepStats)."""
        return self._sweep(self.lib.mdz_rheo_sweep, model, mat, fields, final_update, mem, flags, check)

    def sweep_aniso(self, model, mat, fields, final_update=0, mem=MEM_HOST, flags=0, check=True):
        """NonNewtonianViscosityGridAniso on `fields`.  Returns (status, SweepStats)."""
        return self._sweep(self.lib.mdz_rheo_sweep_aniso, model, mat, fields, final_update, mem,
                           flags, check)

    def sync(self):
        st = SweepStats()
        rc = self.lib.mdz_rheo_sync(self.handle, C.byref(st))
        return rc, st

    def points(self, model, mat, pin, pout, n, aniso=0, mem=MEM_HOST):
        return self.lib.mdz_rheo_points(self.handle, C.byref(model), C.byref(mat), C.byref(pin),
                                        C.byref(pout), n, aniso, mem)

    # ---- viscosity tensors of the momentum equations
    def operators(self, model, mat, fields, ops: dict, jacobian=1, compressible=0, aniso=False, mem=MEM_HOST,
                  flags=0, check=True):
        """RheologicalOperators into the D arrays of `ops` (numpy or device tensors, as `mem`)."""
        st = SweepStats()
        o = make_operator_fields(ops)
        rc = self.lib.mdz_rheo_operators(self.handle, C.byref(model), C.byref(mat), C.byref(fields.struct),
                                         C.byref(o), jacobian, compressible, int(aniso), mem, flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_operators")
        return rc, st

    def strain_rates(self, model, dx, dz, sr: dict, out_of_plane=0, compressible=0.0, mem=MEM_HOST, flags=0,
                     check=True):
        """StrainRateComponents: `sr` holds u_in, v_in, BCp_type, BCg_type and the ten
        output arrays (numpy or device tensors, as `mem`)."""
        st = SweepStats()
        o = make_strain_rate_fields(sr)
        rc = self.lib.mdz_rheo_strain_rates(self.handle, C.byref(model), dx, dz, out_of_plane, float(compressible),
                                            C.byref(o), mem, flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_strain_rates")
        return rc, st

    def softening(self, model, pmat, fields: "PrepFieldSet", smooth_softening=0, hardening_modulus=0,
                  marker_noise=0, mem=MEM_HOST, flags=0, check=True):
        """CohesionFrictionDilationGrid after its marker interpolation (mdz_rheo_softening)."""
        st = SweepStats()
        rc = self.lib.mdz_rheo_softening(self.handle, C.byref(model), C.byref(pmat), C.byref(fields.struct),
                                         smooth_softening, hardening_modulus, marker_noise, mem, flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_softening")
        return rc, st

    def shear_modulus(self, model, pmat, fields: "PrepFieldSet", mem=MEM_HOST, flags=0, check=True):
        """ShearModCompExpGrid (mdz_rheo_shear_modulus)."""
        st = SweepStats()
        rc = self.lib.mdz_rheo_shear_modulus(self.handle, C.byref(model), C.byref(pmat), C.byref(fields.struct), mem,
                                             flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_shear_modulus")
        return rc, st

    def marker_stress(self, model, opts, grid: dict, markers: dict, dx, dz, mem=MEM_HOST, flags=0, check=True):
        """UpdateParticleStress (mdz_rheo_marker_stress): updates the marker stresses (and
        directors) of `markers` and wxz of `grid` in place."""
        st = SweepStats()
        g, m = make_marker_structs(grid, markers, dx, dz)
        rc = self.lib.mdz_rheo_marker_stress(self.handle, C.byref(model), C.byref(opts), C.byref(g), C.byref(m), mem,
                                             flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_marker_stress")
        return rc, st

    def p2mastah(self, model, grid: dict, markers: dict, values, avg, stencil, node_n, node_s, dx, dz,
                 mem=MEM_HOST, flags=0, check=True):
        """P2Mastah of a marker array onto centroids (node_n) and/or vertices (node_s),
        updated in place (mdz_rheo_p2mastah)."""
        st = SweepStats()
        g, m = make_marker_structs(grid, markers, dx, dz)
        rc = self.lib.mdz_rheo_p2mastah(self.handle, C.byref(model), C.byref(g), C.byref(m), _ptr(values), avg,
                                        stencil, _ptr(node_n), _ptr(node_s), mem, flags, C.byref(st))
        if check and rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_p2mastah")
        return rc, st

    # ---- launch-shape autotuner
    # (threads per block, waves of resident CTAs or 0 for one thread per node, form); forms:
    # 0 the 128-register kernel, 1 the 255-register kernel, 2 persistent work counter,
    # 3 the compacting kernel (isotropic; one thread per node for the anisotropic sweep)
    AUTOTUNE_CANDIDATES = ([(b, w, 0) for b in (128, 64) for w in (0, 1, 2, 4, 8)]
                           + [(128, 0, 1), (128, 1, 2), (128, 0, 3)])
    AUTOTUNE_NAMES = ([f"block {b}, " + (f"{w} waves" if w else "one thread per node") for b in (128, 64)
                       for w in (0, 1, 2, 4, 8)] + ["block 128, one thread per node, 255 registers (2 CTAs/SM)",
                                                    "block 128, persistent warps on a work counter",
                                                    "block 128, yielding items compacted per CTA"])

    def autotune(self, model, mat, fields, aniso=False, flags=0, reps=3):
        """Time every launch shape on this device-resident grid and keep the fastest.
        Returns (ms per candidate, index of the best, (block, grid_cap) now in use)."""
        ms = np.zeros(len(self.AUTOTUNE_CANDIDATES))
        best = C.c_int()
        rc = self.lib.mdz_rheo_autotune(self.handle, C.byref(model), C.byref(mat), C.byref(fields.struct),
                                        int(aniso), flags, reps, ms.ctypes.data, C.byref(best))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_autotune")
        return ms, best.value, self.launch_shape(aniso)

    def launch_form(self, aniso=False):
        f = C.c_int()
        rc = self.lib.mdz_rheo_get_launch_form(self.handle, int(aniso), C.byref(f))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_get_launch_form")
        return f.value

    def set_launch_shape(self, aniso=False, block=128, grid_cap=0, form=0):
        rc = self.lib.mdz_rheo_set_launch_shape(self.handle, int(aniso), block, grid_cap, form)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_set_launch_shape")

    def launch_shape(self, aniso=False):
        b, g = C.c_int(), C.c_int()
        rc = self.lib.mdz_rheo_get_launch_shape(self.handle, int(aniso), C.byref(b), C.byref(g))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_get_launch_shape")
        return b.value, g.value

    # ---- learned warm start
    def set_warmstart(self, w: Optional[MlpWeights], polish_iters: int = DEFAULT_START):
        rc = self.lib.mdz_rheo_set_warmstart(self.handle, None if w is None else C.byref(w), polish_iters)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_set_warmstart")

    def set_mma_poll_limit(self, limit: int):
        """Test hook: polls of each tcgen05 completion wait before giving up (0: at once; negative: the
        default)."""
        rc = self.lib.mdz_rheo_set_mma_poll_limit(self.handle, limit)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_set_mma_poll_limit")

    def collect(self, model, mat, fields, X, Y, aniso=False, final_update=0, mem=MEM_HOST):
        """A sweep that also records per-(phase, node) features X [items, 16] and targets Y [items, 2]."""
        st = SweepStats()
        rc = self.lib.mdz_rheo_collect(self.handle, C.byref(model), C.byref(mat), C.byref(fields.struct),
                                       final_update, int(aniso), mem, _ptr(X), _ptr(Y), C.byref(st))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_collect")
        return st

    def train_mlp(self, X, Y, n_feat, cfg: MlpTrainCfg, w: Optional[MlpWeights] = None, mem=MEM_HOST):
        w = MlpWeights() if w is None else w
        loss = np.zeros(cfg.epochs, np.float32)
        rc = self.lib.mdz_rheo_train_mlp(self.handle, _ptr(X), _ptr(Y), int(Y.shape[0]), n_feat, C.byref(cfg),
                                         C.byref(w), loss.ctypes.data, mem)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_train_mlp")
        return w, loss

    def mlp_predict(self, w: MlpWeights, X, mem=MEM_HOST):
        n = int(X.shape[0])
        Yp = np.zeros((n, 2), np.float32)
        rc = self.lib.mdz_rheo_mlp_predict(self.handle, C.byref(w), _ptr(X), Yp.ctypes.data, n, mem)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_mlp_predict")
        return Yp

    def mlp_gradient(self, w: MlpWeights, X, Y, w_pl=1.0, mem=MEM_HOST):
        g = MlpWeights()
        loss = np.zeros(2, np.float32)
        rc = self.lib.mdz_rheo_mlp_gradient(self.handle, C.byref(w), _ptr(X), _ptr(Y), int(Y.shape[0]), w_pl,
                                            C.byref(g), loss.ctypes.data, mem)
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_mlp_gradient")
        return g, loss

    def get_iterations(self, out_n: np.ndarray, out_s: np.ndarray):
        rc = self.lib.mdz_rheo_get_iterations(self.handle, _ptr(out_n), _ptr(out_s))
        if rc != MDZ_OK:
            raise RheoError(rc, "mdz_rheo_get_iterations")
