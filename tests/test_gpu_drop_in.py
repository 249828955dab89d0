"""The MDOODZ-side drop-in over the GPU library, against the reference's own functions.

mdoodz7.0_gb300/host/mdz_rheo_mdoodz.c defines NonNewtonianViscosityGrid(Aniso) and
StrainRateComponents with the reference's signatures (mdoodz-private.h:423, :437) and
forwards them to libmdz_rheo_gb300.so through the C ABI.  oracle/_ref/libmdz_gpushim.so
links that translation unit, unchanged, with the real GPU library and with the
reference's own sources (its functions renamed, so both sit side by side), and the
reference's harness builds a real `grid` / `mat_prop` / `params` / `scale` from the
test's arrays.  So this is a whole MDOODZ call on the GPU, compared with the same call
of the reference itself, within the parity bar of the other GPU tests.  The library is built by `__graft_entry__.build()` from the
reference's sources, or from their preprocessed units where the tree is absent.
"""
import numpy as np
import pytest

import mdz_rheo as R
import mdz_workloads as W
import oracle_lib as O
from common import RTOL, clone, worst

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(O.gpushim() is None, reason="GPU drop-in library not built (no reference units)")]

CASES = {
    "plain_small": (lambda: W.plain_small(seed=0, ncx=61), False, 0),
    "plain_large": (lambda: W.plain_large(seed=1, ncx=80, ncz=72), False, 0),
    "plain_large_final_update": (lambda: W.plain_large(seed=2, ncx=65), False, 1),
    "plain_large_harmonic_typical": (lambda: W.plain_large(seed=3, ncx=48, sc=W.TYPICAL, eta_average=1), False, 0),
    "aniso": (lambda: W.aniso(seed=4, ncx=64), True, 0),
}


def compare(a, b, w, label):
    errs = worst(a, b, w.arrays, w.model)
    bad = {k: v for k, v in errs.items() if v > RTOL}
    print(label, "max scaled error", max(errs.values()))
    assert not bad, f"{label}: {bad}"


@pytest.mark.parametrize("name", list(CASES))
def test_drop_in_on_gpu_matches_reference(name):
    make, aniso, fu = CASES[name]
    w = make()
    ref, gpu = clone(w.arrays), clone(w.arrays)
    assert O.gpushim_sweep(w.model, w.mat, R.FieldSet(ref), fu, aniso, drop_in=False) == 0
    assert O.gpushim_sweep(w.model, w.mat, R.FieldSet(gpu), fu, aniso, drop_in=True) == 0
    compare(gpu, ref, w, f"drop-in {name}")


def test_drop_in_on_gpu_periodic_and_air():
    w = W.plain_large(seed=5, ncx=48)
    w.model.periodic_x = 1
    w.arrays["BCp_type"][-96:] = 30
    w.arrays["BCg_type"][-49 * 3:] = 30
    ref, gpu = clone(w.arrays), clone(w.arrays)
    assert O.gpushim_sweep(w.model, w.mat, R.FieldSet(ref), 0, False, drop_in=False) == 0
    assert O.gpushim_sweep(w.model, w.mat, R.FieldSet(gpu), 0, False, drop_in=True) == 0
    compare(gpu, ref, w, "drop-in periodic + air")


def test_drop_in_strain_rates_on_gpu():
    """StrainRateComponents through the drop-in on the GPU against the reference's own,
    within 1e-13 of each field's largest magnitude.  (The GPU kernel reproduces the
    reference's x86-64 build bit for bit -- tests/test_gpu_strain_rates.py, on the golden
    fixtures -- but where the reference is compiled on an aarch64 host, gcc contracts its
    multiply-adds into fused ones by default, which moves its own last bits.)"""
    v = W.velocity_field(seed=12, ncx=70, ncz=50, air=0.2, periodic=1)
    ref = {k: a.copy() for k, a in v.arrays.items()}
    gpu = {k: a.copy() for k, a in v.arrays.items()}
    assert O.gpushim_strain_rates(v.model, v.info["dx"], v.info["dz"], ref, 1, 1.0, drop_in=False) == 0
    assert O.gpushim_strain_rates(v.model, v.info["dx"], v.info["dz"], gpu, 1, 1.0, drop_in=True) == 0
    for k in R.SR_N + R.SR_S:
        scale = max(float(np.max(np.abs(ref[k]))), 1e-300)
        err = float(np.max(np.abs(gpu[k] - ref[k]))) / scale
        assert err <= 1e-13, (k, err)
