"""ctypes loader for the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, as the checker.  Two libraries can be loaded:

  * build/librheo_oracle.so -- the C restatement (rheo_oracle.c), built on any
    host by `make -C oracle`;
  * _ref/libmdz_ref.so      -- MDOODZ7.0's own sources plus ref_harness.c,
    built by `make -C oracle ref` where the reference tree is present;
  * _ref/libmdz_shimtest.so -- the MDOODZ-side drop-in (host/mdz_rheo_mdoodz.c)
    over a CPU backend, beside the reference's own sweep (`make -C oracle shim`).

Both take the same plain-pointer structs as the GPU library (include/mdz_rheo.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "mdoodz7.0_gb300"))
import mdz_rheo as R  # noqa: E402

ORACLE_SO = os.path.join(HERE, "build", "librheo_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmdz_ref.so")
SHIM_SO = os.path.join(HERE, "_ref", "libmdz_shimtest.so")
# The MDOODZ7.0 source tree the pinning build compiles: MDZ_REFERENCE_TREE, else a
# checkout named `reference` beside this repository.  Absent (as on a machine that only
# runs the GPU tests), only the restatement is built.
REF_TREE = os.environ.get("MDZ_REFERENCE_TREE") or os.path.join(os.path.dirname(REPO), "reference")


GPUSHIM_SO = os.path.join(HERE, "_ref", "libmdz_gpushim.so")
PRE_DIR = os.path.join(HERE, "_ref", "pre")
GPU_LIB = os.path.join(REPO, "mdoodz7.0_gb300", "build", "libmdz_rheo_gb300.so")


def build(ref: bool = False, quiet: bool = True):
    """Build the restatement and, when asked, the reference's own code (_ref): from the
    MDOODZ7.0 tree where it exists (which also writes the preprocessed units), else from
    the preprocessed units written there before."""
    targets, tree = ["all"], ""
    if ref and os.path.isdir(os.path.join(REF_TREE, "MDLIB")):
        targets += ["pre", "ref", "shim"]
        tree = REF_TREE
    elif ref and os.path.exists(os.path.join(PRE_DIR, "RheologyDensity.i")):
        targets += ["ref", "shim"]
    if len(targets) > 1 and os.path.exists(GPU_LIB):
        targets.append("gpushim")
    out = subprocess.run(["make", "-C", HERE, f"REF={tree}", "-j8"] + targets,
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _bind(lib, prefix):
    for name in ("sweep", "sweep_aniso"):
        fn = getattr(lib, f"{prefix}_{name}", None)
        if fn is None:
            continue
        if prefix == "orc":
            fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.GridFields), C.c_int,
                           C.c_void_p, C.c_void_p, C.POINTER(R.SweepStats)]
        fn.restype = C.c_int
    ops = getattr(lib, f"{prefix}_operators", None)
    if ops is not None:
        ops.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.GridFields),
                        C.POINTER(R.OperatorFields), C.c_int, C.c_int, C.c_int]
        ops.restype = C.c_int
    pts = getattr(lib, f"{prefix}_points")
    pts.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.PointInputs),
                    C.POINTER(R.PointOutputs), C.c_int64, C.c_int]
    pts.restype = C.c_int
    return lib


_orc = None
_ref = None


def oracle():
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = C.CDLL(ORACLE_SO)
        _bind(lib, "orc")
        lib.orc_interp_c2v.argtypes = [C.POINTER(R.Model), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.orc_num_threads.restype = C.c_int
        _orc = lib
    return _orc


def reference():
    """The reference's own code, or None where it was not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        lib = C.CDLL(REF_SO)
        lib.ref_sweep.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.GridFields),
                                  C.c_int, C.c_int]
        lib.ref_sweep.restype = C.c_int
        _bind(lib, "ref")
        _ref = lib
    return _ref


def orc_sweep(model, mat, fs: "R.FieldSet", final_update=0, aniso=False, iters_n=None, iters_s=None):
    lib = oracle()
    st = R.SweepStats()
    fn = lib.orc_sweep_aniso if aniso else lib.orc_sweep
    rc = fn(C.byref(model), C.byref(mat), C.byref(fs.struct), final_update,
            None if iters_n is None else iters_n.ctypes.data,
            None if iters_s is None else iters_s.ctypes.data, C.byref(st))
    return rc, st


def ref_sweep(model, mat, fs: "R.FieldSet", final_update=0, aniso=False):
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    return lib.ref_sweep(C.byref(model), C.byref(mat), C.byref(fs.struct), final_update, int(aniso))


_shim = None


def shimtest():
    """The drop-in check library, or None where it was not built."""
    global _shim
    if _shim is None and os.path.exists(SHIM_SO):
        lib = C.CDLL(SHIM_SO)
        for name in ("shimtest_ref_sweep", "shimtest_shim_sweep"):
            fn = getattr(lib, name)
            fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.GridFields), C.c_int, C.c_int]
            fn.restype = C.c_int
        for name in ("shimtest_ref_operators", "shimtest_shim_operators"):
            fn = getattr(lib, name)
            fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.GridFields),
                           C.POINTER(R.OperatorFields), C.c_int, C.c_int, C.c_int]
            fn.restype = C.c_int
        _shim = lib
    return _shim


_gpushim = None


def gpushim():
    """The drop-in over the GPU library beside the reference's own code, or None where it
    was not built."""
    global _gpushim
    if _gpushim is None and os.path.exists(GPUSHIM_SO):
        lib = C.CDLL(GPUSHIM_SO)
        for name in ("shimtest_ref_sweep", "shimtest_shim_sweep"):
            fn = getattr(lib, name)
            fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.Materials), C.POINTER(R.GridFields), C.c_int, C.c_int]
            fn.restype = C.c_int
        _gpushim = lib
    return _gpushim


def gpushim_sweep(model, mat, fs: "R.FieldSet", final_update=0, aniso=False, drop_in=True):
    """NonNewtonianViscosityGrid(Aniso) on a harness-built `grid`: the drop-in over the GPU
    library (drop_in=True) or the reference's own."""
    lib = gpushim()
    fn = lib.shimtest_shim_sweep if drop_in else lib.shimtest_ref_sweep
    return fn(C.byref(model), C.byref(mat), C.byref(fs.struct), final_update, int(aniso))


def gpushim_strain_rates(model, dx, dz, sr: dict, out_of_plane=0, compressible=0.0, drop_in=True):
    """StrainRateComponents on a harness-built `grid`: the drop-in over the GPU library or
    the reference's own."""
    name = "shimtest_shim_strain_rates" if drop_in else "shimtest_ref_strain_rates"
    return _strain_fn(gpushim(), name)(C.byref(model), dx, dz, out_of_plane, float(compressible),
                                       C.byref(R.make_strain_rate_fields(sr)))


def shim_sweep(model, mat, fs: "R.FieldSet", final_update=0, aniso=False, drop_in=True):
    """NonNewtonianViscosityGrid(Aniso) on a harness-built `grid`: the drop-in's
    (drop_in=True) or the reference's own."""
    lib = shimtest()
    fn = lib.shimtest_shim_sweep if drop_in else lib.shimtest_ref_sweep
    return fn(C.byref(model), C.byref(mat), C.byref(fs.struct), final_update, int(aniso))


def orc_operators(model, mat, fs: "R.FieldSet", ops: dict, jacobian=1, compressible=0, aniso=False):
    """RheologicalOperators on the restatement; `ops` is a dict of numpy D arrays."""
    o = R.make_operator_fields(ops)
    return oracle().orc_operators(C.byref(model), C.byref(mat), C.byref(fs.struct), C.byref(o), jacobian,
                                  compressible, int(aniso))


def ref_operators(model, mat, fs: "R.FieldSet", ops: dict, jacobian=1, compressible=0, aniso=False):
    """RheologicalOperators of the reference build."""
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    o = R.make_operator_fields(ops)
    return lib.ref_operators(C.byref(model), C.byref(mat), C.byref(fs.struct), C.byref(o), jacobian,
                             compressible, int(aniso))


def shim_operators(model, mat, fs: "R.FieldSet", ops: dict, jacobian=1, compressible=0, aniso=False,
                   drop_in=True):
    """RheologicalOperators on a harness-built `grid`: the drop-in's or the reference's."""
    lib = shimtest()
    fn = lib.shimtest_shim_operators if drop_in else lib.shimtest_ref_operators
    return fn(C.byref(model), C.byref(mat), C.byref(fs.struct), C.byref(R.make_operator_fields(ops)), jacobian,
              compressible, int(aniso))


def _strain_fn(lib, name):
    fn = getattr(lib, name)
    fn.argtypes = [C.POINTER(R.Model), C.c_double, C.c_double, C.c_int, C.c_double, C.POINTER(R.StrainRateFields)]
    fn.restype = C.c_int
    return fn


def orc_strain_rates(model, dx, dz, sr: dict, out_of_plane=0, compressible=0.0):
    """StrainRateComponents on the restatement; `sr` is a dict of numpy arrays."""
    return _strain_fn(oracle(), "orc_strain_rates")(C.byref(model), dx, dz, out_of_plane, float(compressible),
                                                    C.byref(R.make_strain_rate_fields(sr)))


def ref_strain_rates(model, dx, dz, sr: dict, out_of_plane=0, compressible=0.0):
    """StrainRateComponents of the reference build."""
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    return _strain_fn(lib, "ref_strain_rates")(C.byref(model), dx, dz, out_of_plane, float(compressible),
                                               C.byref(R.make_strain_rate_fields(sr)))


def shim_strain_rates(model, dx, dz, sr: dict, out_of_plane=0, compressible=0.0, drop_in=True):
    """StrainRateComponents on a harness-built `grid`: the drop-in's or the reference's."""
    name = "shimtest_shim_strain_rates" if drop_in else "shimtest_ref_strain_rates"
    return _strain_fn(shimtest(), name)(C.byref(model), dx, dz, out_of_plane, float(compressible),
                                        C.byref(R.make_strain_rate_fields(sr)))


def orc_softening(model, pmat, fs: "R.PrepFieldSet", smooth_softening=0, hardening_modulus=0, marker_noise=0):
    fn = oracle().orc_softening
    fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.PrepMaterials), C.POINTER(R.PrepFields), C.c_int, C.c_int, C.c_int]
    return fn(C.byref(model), C.byref(pmat), C.byref(fs.struct), smooth_softening, hardening_modulus, marker_noise)


def orc_shear_modulus(model, pmat, fs: "R.PrepFieldSet"):
    fn = oracle().orc_shear_modulus
    fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.PrepMaterials), C.POINTER(R.PrepFields)]
    return fn(C.byref(model), C.byref(pmat), C.byref(fs.struct))


def _markers_call(fn, model, pmat, fs, mk, smooth_softening, hardening_modulus, marker_noise):
    import numpy as np
    fn.argtypes = ([C.POINTER(R.Model), C.POINTER(R.PrepMaterials), C.POINTER(R.PrepFields), C.c_int64]
                   + [C.c_void_p] * 4 + [C.c_double] * 4 + [C.c_int] * 4 + [C.c_void_p] * 2)
    nc, nv = (model.Nx - 1) * (model.Nz - 1), model.Nx * model.Nz
    sn, ss = np.zeros(nc), np.zeros(nv)
    rc = fn(C.byref(model), C.byref(pmat), C.byref(fs.struct), mk["x"].size, mk["x"].ctypes.data,
            mk["z"].ctypes.data, mk["phase"].ctypes.data, mk["strain_pl"].ctypes.data, mk["xmin"], mk["zmin"],
            mk["dx"], mk["dz"], mk["interp_stencil"], smooth_softening, hardening_modulus, marker_noise,
            sn.ctypes.data, ss.ctypes.data)
    return rc, sn, ss


def ref_softening_markers(model, pmat, fs: "R.PrepFieldSet", mk: dict, smooth_softening=0, hardening_modulus=0,
                          marker_noise=0):
    """The reference's CohesionFrictionDilationGrid with markers `mk` (x, z, phase, strain_pl,
    xmin, zmin, dx, dz, interp_stencil); returns (rc, strain_pl_n, strain_pl_s) -- the plastic
    strain its P2Mastah put on the grid."""
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    return _markers_call(lib.ref_softening_markers, model, pmat, fs, mk, smooth_softening, hardening_modulus,
                         marker_noise)


def shim_softening_markers(model, pmat, fs: "R.PrepFieldSet", mk: dict, smooth_softening=0, hardening_modulus=0,
                           marker_noise=0, drop_in=True):
    name = "shimtest_shim_softening_markers" if drop_in else "shimtest_ref_softening_markers"
    return _markers_call(getattr(shimtest(), name), model, pmat, fs, mk, smooth_softening, hardening_modulus,
                         marker_noise)


def ref_shear_modulus(model, pmat, fs: "R.PrepFieldSet"):
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    fn = lib.ref_shear_modulus
    fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.PrepMaterials), C.POINTER(R.PrepFields)]
    return fn(C.byref(model), C.byref(pmat), C.byref(fs.struct))


def shim_shear_modulus(model, pmat, fs: "R.PrepFieldSet", drop_in=True):
    fn = getattr(shimtest(), "shimtest_shim_shear_modulus" if drop_in else "shimtest_ref_shear_modulus")
    fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.PrepMaterials), C.POINTER(R.PrepFields)]
    return fn(C.byref(model), C.byref(pmat), C.byref(fs.struct))


def _marker_call(fn, model, opts, grid, markers, dx, dz):
    fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.MarkerOpts), C.POINTER(R.MarkerGrid), C.POINTER(R.Markers)]
    fn.restype = C.c_int
    g, m = R.make_marker_structs(grid, markers, dx, dz)
    return fn(C.byref(model), C.byref(opts), C.byref(g), C.byref(m))


def orc_marker_stress(model, opts, grid: dict, markers: dict, dx, dz):
    """UpdateParticleStress on the restatement (numpy arrays, updated in place)."""
    return _marker_call(oracle().orc_marker_stress, model, opts, grid, markers, dx, dz)


def ref_marker_stress(model, opts, grid: dict, markers: dict, dx, dz):
    """The reference's UpdateParticleStress (numpy arrays, updated in place)."""
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    return _marker_call(lib.ref_marker_stress, model, opts, grid, markers, dx, dz)


def shim_marker_stress(model, opts, grid: dict, markers: dict, dx, dz, drop_in=True):
    name = "shimtest_shim_marker_stress" if drop_in else "shimtest_ref_marker_stress"
    return _marker_call(getattr(shimtest(), name), model, opts, grid, markers, dx, dz)


def _p2m_call(fn, model, grid, markers, values, avg, stencil, node_n, node_s, dx, dz):
    fn.argtypes = [C.POINTER(R.Model), C.POINTER(R.MarkerGrid), C.POINTER(R.Markers), C.c_void_p, C.c_int, C.c_int,
                   C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    g, m = R.make_marker_structs(grid, markers, dx, dz)
    return fn(C.byref(model), C.byref(g), C.byref(m), R._ptr(values), avg, stencil, R._ptr(node_n), R._ptr(node_s))


def orc_p2mastah(model, grid: dict, markers: dict, values, avg, stencil, node_n, node_s, dx, dz):
    """P2Mastah of a marker array on the restatement (node arrays updated in place)."""
    return _p2m_call(oracle().orc_p2mastah, model, grid, markers, values, avg, stencil, node_n, node_s, dx, dz)


def ref_p2mastah(model, grid: dict, markers: dict, values, avg, stencil, node_n, node_s, dx, dz):
    """The reference's P2Mastah of a marker array, on one thread (node arrays updated in place)."""
    lib = reference()
    if lib is None:
        raise RuntimeError("reference library not built (oracle/_ref)")
    return _p2m_call(lib.ref_p2mastah, model, grid, markers, values, avg, stencil, node_n, node_s, dx, dz)


def orc_points(model, mat, pin, pout, n, aniso=0):
    return oracle().orc_points(C.byref(model), C.byref(mat), C.byref(pin), C.byref(pout), n, aniso)


def ref_points(model, mat, pin, pout, n, aniso=0):
    return reference().ref_points(C.byref(model), C.byref(mat), C.byref(pin), C.byref(pout), n, aniso)
