"""Generate the golden fixtures from MDOODZ7.0's own code.

Runs the reference's NonNewtonianViscosityGrid(Aniso), RheologicalOperators (on the
fields the sweep produced), StrainRateComponents, CohesionFrictionDilationGrid (with
markers), ShearModCompExpGrid, UpdateParticleStress and ViscosityConcise(Aniso), compiled from the MDOODZ7.0
sources by oracle/Makefile (target `ref`), on the cases of cases.py and stores their
outputs in tests/golden/*.npz.  Inputs are
regenerated from the seeds by the tests; a SHA-256 of the inputs is stored
beside the outputs so that a change in the generators is caught.

    python tests/golden/make_golden.py        (needs the reference tree)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "mdoodz7.0_gb300"), os.path.join(REPO, "oracle"), HERE]

import cases  # noqa: E402
import mdz_rheo as R  # noqa: E402
import oracle_lib as O  # noqa: E402

INPUT_GRID = [k for k in R.CEN_IN + R.VER_IN + R.ANI_IN_N + R.ANI_IN_S + ["BCp_type", "BCg_type"]]
STRAIN_INPUTS = ["u_in", "v_in", "BCp_type", "BCg_type", "wxz"]
PREP_INPUTS = ["phase_perc_n", "phase_perc_s", "BCp_type", "BCg_type", "strain_pl_n", "strain_pl_s", "noise_n",
               "noise_s"]


def digest(arrays, keys):
    h = hashlib.sha256()
    for k in keys:
        v = arrays.get(k)
        if v is None:
            continue
        for x in (v if isinstance(v, list) else [v]):
            h.update(np.ascontiguousarray(x).tobytes())
    return h.hexdigest()


def grid_inputs_digest(w):
    return digest(w.arrays, INPUT_GRID + ["phase_perc_n", "phase_perc_s"])


def prep_inputs_digest(w):
    """Grid inputs and materials of a preparation case (and its markers, if any)."""
    h = hashlib.sha256(digest(w.arrays, PREP_INPUTS).encode())
    h.update(bytes(w.mat))
    for k in ("x", "z", "phase", "strain_pl"):
        if "markers" in w.info:
            h.update(np.ascontiguousarray(w.info["markers"][k]).tobytes())
    return h.hexdigest()


def prep_inputs(w):
    """The inputs of a preparation case, stored beside its outputs: the fixture then needs
    no generator (numpy's transcendental functions differ between hosts in the last bits,
    and these cases run on hosts other than the one that made them)."""
    out = {k: np.array(w.arrays[k]) for k in PREP_INPUTS if not k.startswith("phase_")}
    for k in ("phase_perc_n", "phase_perc_s"):
        out[k] = np.stack(w.arrays[k])
    out["model_bytes"] = np.frombuffer(bytes(w.model), np.uint8)
    out["materials_bytes"] = np.frombuffer(bytes(w.mat), np.uint8)
    return out


def load_prep_inputs(g):
    """(model, materials, arrays) of a preparation fixture, outputs set to a sentinel."""
    model = R.Model.from_buffer_copy(g["model_bytes"].tobytes())
    mat = R.PrepMaterials.from_buffer_copy(g["materials_bytes"].tobytes())
    a = {k: np.array(g[k]) for k in PREP_INPUTS if not k.startswith("phase_")}
    for k in ("phase_perc_n", "phase_perc_s"):
        a[k] = [np.ascontiguousarray(x) for x in g[k]]
    nc, nv = (model.Nx - 1) * (model.Nz - 1), model.Nx * model.Nz
    for k in R.SOFT_N + R.MOD_N:
        a[k] = np.full(nc, -7.0)
    for k in R.SOFT_S + R.MOD_S:
        a[k] = np.full(nv, -7.0)
    return model, mat, a


def marker_opts(elastic, rot, aniso, adv, stencil, subgrid=0, G=None):
    o = R.MarkerOpts()
    o.elastic, o.subgrid_diffusion, o.stress_rotation = elastic, subgrid, rot
    o.anisotropy, o.advection, o.interp_stencil = aniso, adv, stencil
    if G is not None:
        o.set_G(G)
    return o


def marker_inputs(w):
    """The inputs of a marker case, stored beside the reference's outputs."""
    out = {"grid_" + k: np.array(v) for k, v in w.arrays.items()}
    out.update({"mk_" + k: np.array(v) for k, v in w.info["markers"].items()})
    out["model_bytes"] = np.frombuffer(bytes(w.model), np.uint8)
    out["spacing"] = np.array([w.info["dx"], w.info["dz"]])
    out["mat_G"] = np.array(w.info["G"])
    return out


def load_marker_G(g):
    """The per-phase shear modulus of a marker fixture (None for fixtures without one)."""
    return np.array(g["mat_G"]) if "mat_G" in g.files else None


def load_marker_inputs(g):
    """(model, grid arrays, marker arrays, dx, dz) of a marker fixture."""
    model = R.Model.from_buffer_copy(g["model_bytes"].tobytes())
    grid = {k[5:]: np.array(g[k]) for k in g.files if k.startswith("grid_")}
    mk = {k[3:]: np.array(g[k]) for k in g.files if k.startswith("mk_")}
    return model, grid, mk, float(g["spacing"][0]), float(g["spacing"][1])


def point_inputs_digest(pin):
    return digest(pin, ["phase"] + R.PT_IN + R.PT_ANI)


def grid_outputs(arrays):
    out = {}
    for k in R.VER_INTERP + R.CEN_OUT + R.VER_OUT:
        if k in arrays:
            out[k] = arrays[k]
    for k in ("phase_eta_n", "phase_eta_s"):
        out[k] = np.stack(arrays[k])
    return out


def main(only=()):
    """Every fixture group, or only the groups named (grid, operators, strain_rates,
    softening, shear_modulus, markers, points)."""
    O.build(ref=True)
    if O.reference() is None:
        sys.exit("the reference tree is needed to generate golden fixtures")
    for name, (builder, aniso, fu) in cases.GRID_CASES.items():
        if only and "grid" not in only:
            break
        w = builder()
        dig = grid_inputs_digest(w)
        a = {k: ([x.copy() for x in v] if isinstance(v, list) else v.copy()) for k, v in w.arrays.items()}
        O.ref_sweep(w.model, w.mat, R.FieldSet(a), final_update=fu, aniso=aniso)
        np.savez_compressed(os.path.join(HERE, f"grid_{name}.npz"), inputs_sha256=dig, **grid_outputs(a))
        print("grid", name, w.nodes, "nodes")
    for name, (grid_case, jac, comp) in cases.OPERATOR_CASES.items():
        if only and "operators" not in only:
            break
        builder, aniso, fu = cases.GRID_CASES[grid_case]
        w = builder()
        O.ref_sweep(w.model, w.mat, R.FieldSet(w.arrays), final_update=fu, aniso=aniso)
        ops = R.alloc_operator_fields(w.Nc, w.Nv)
        O.ref_operators(w.model, w.mat, R.FieldSet(w.arrays), ops, jac, comp, aniso)
        np.savez_compressed(os.path.join(HERE, f"operators_{name}.npz"), inputs_sha256=grid_inputs_digest(builder()),
                            **ops)
        print("operators", name)
    for name, (builder, oop, comp) in cases.STRAIN_CASES.items():
        if only and "strain_rates" not in only:
            break
        w = builder()
        dig = digest(w.arrays, STRAIN_INPUTS)
        O.ref_strain_rates(w.model, w.info["dx"], w.info["dz"], w.arrays, oop, comp)
        np.savez_compressed(os.path.join(HERE, f"strain_rates_{name}.npz"), inputs_sha256=dig,
                            **{k: w.arrays[k] for k in R.SR_N + R.SR_S})
        print("strain rates", name)
    for name, (builder, smooth, hard, noise, stencil) in cases.SOFTENING_CASES.items():
        if only and "softening" not in only:
            break
        w = builder()
        mk = dict(w.info["markers"], interp_stencil=stencil)
        dig = prep_inputs_digest(w)
        inputs = prep_inputs(w)
        rc, sn, ss = O.ref_softening_markers(w.model, w.mat, R.PrepFieldSet(w.arrays), mk, smooth, hard, noise)
        inputs.update(strain_pl_n=sn, strain_pl_s=ss)
        np.savez_compressed(os.path.join(HERE, f"softening_{name}.npz"), inputs_sha256=dig, **inputs,
                            **{k: w.arrays[k] for k in R.SOFT_N + R.SOFT_S})
        print("softening", name)
    for name, builder in cases.SHEAR_CASES.items():
        if only and "shear_modulus" not in only:
            break
        w = builder()
        dig = prep_inputs_digest(w)
        inputs = prep_inputs(w)
        O.ref_shear_modulus(w.model, w.mat, R.PrepFieldSet(w.arrays))
        np.savez_compressed(os.path.join(HERE, f"shear_modulus_{name}.npz"), inputs_sha256=dig, **inputs,
                            **{k: w.arrays[k] for k in R.MOD_N + R.MOD_S})
        print("shear modulus", name)
    for name, (builder, *o) in cases.MARKER_CASES.items():
        if only and "markers" not in only:
            break
        w = builder()
        opts = marker_opts(*o, G=w.info["G"])
        inputs = marker_inputs(w)
        grid = {k: w.arrays[k].copy() for k in w.arrays}
        mk = {k: v.copy() for k, v in w.info["markers"].items()}
        O.ref_marker_stress(w.model, opts, grid, mk, w.info["dx"], w.info["dz"])
        np.savez_compressed(os.path.join(HERE, f"markers_{name}.npz"), **inputs,
                            **{"out_" + k: mk[k] for k in ("sxxd", "szzd", "sxz", "nx", "nz")}, out_wxz=grid["wxz"])
        print("markers", name)
    for name in cases.POINT_CASES:
        if only and "points" not in only:
            break
        md, m, pin, aniso, centroid, fu = cases.point_case(name)
        n = pin["phase"].size
        out = cases.alloc_point_outputs(n)
        pi, po = R.make_points(pin, out, centroid=centroid, final_update=fu)
        O.ref_points(md, m, pi, po, n, int(aniso))
        keep = {k: out[k] for k in R.PT_OUT}
        np.savez_compressed(os.path.join(HERE, f"points_{name}.npz"), inputs_sha256=point_inputs_digest(pin), **keep)
        print("points", name, n)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
