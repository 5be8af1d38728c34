"""The planner (zr_plan, Engine.plan): measured launch variants of the
transform kernels, saved and restored like FFTW wisdom, that change no
result."""
import ctypes as C
import itertools
import json

import numpy as np
import pytest

from tests import gpu_helpers as gh
from zorro_gb300 import _lib
from zorro_gb300.synthetic import make_movie

pytestmark = pytest.mark.gpu


def _shape(P, C_, mS, nf=6):
    return _lib.PlanShape(P[0], P[1], C_[0], C_[1], mS, nf)


def test_plan_measures_and_installs_a_choice():
    torch = gh.torch_mod()
    lib = _lib.load()
    _lib.call("zr_init", torch.cuda.current_device())
    shape = _shape((512, 512), (256, 256), 20)
    wb = lib.zr_plan_work_bytes(C.byref(shape))
    assert wb > 0
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    choice = _lib.PlanChoice()
    _lib.call("zr_plan", C.byref(shape), work.data_ptr(), wb, gh.stream(), C.byref(choice))
    picked = (choice.fwd_rows, choice.fwd_cols, choice.xc_cols, choice.xc_rows)
    assert all(v in (1, 2, 4) for v in picked), picked
    ms = np.array([list(r) for r in choice.ms_spectra] + [list(r) for r in choice.ms_pairs])
    assert np.all(ms > 0) and np.all(np.isfinite(ms))
    # the fastest candidate is the one installed
    assert choice.ms_spectra[(1, 2, 4).index(choice.fwd_rows)][(1, 2, 4).index(choice.fwd_cols)] == ms[:3].min()
    got = _lib.PlanChoice()
    _lib.call("zr_plan_get", C.byref(shape), C.byref(got))
    assert (got.fwd_rows, got.fwd_cols, got.xc_cols, got.xc_rows) == picked
    bad = _lib.PlanChoice(3, 1, 1, 1)
    assert lib.zr_plan_set(C.byref(shape), C.byref(bad)) == -1
    _lib.call("zr_plan_set", C.byref(shape), C.byref(_lib.PlanChoice(0, 0, 0, 0)))


@pytest.mark.parametrize("P,C_,mS", [((512, 512), (256, 256), 20), ((1536, 1536), (768, 768), 40)])
def test_every_variant_gives_the_same_spectra_and_windows(P, C_, mS):
    """Spectra and correlation windows with each of the 3 x 3 forward and
    3 x 3 correlation variants: bit for bit those of the built-in ones."""
    mv = make_movie(5, (P[0] - 40, P[1] - 60), seed=71, mean_dose=1.5, drift_sigma=1.0)
    shape = _shape(P, C_, mS)
    N = 5
    pairs = [(I, J) for I in range(N) for J in range(I + 1, N)]

    def run(choice):
        _lib.call("zr_plan_set", C.byref(shape), C.byref(choice))
        G, S, GM, _, dev = gh.spectra(mv["images"], P, C_)
        _, cw, _ = gh.windows(dev, N, C_, mS, pairs)
        return G, S, cw

    ref = run(_lib.PlanChoice(0, 0, 0, 0))
    for fr, fc in itertools.product((1, 2, 4), repeat=2):
        got = run(_lib.PlanChoice(fr, fc, 0, 0))
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), (fr, fc)
    for xc, xr in itertools.product((1, 2, 4), repeat=2):
        got = run(_lib.PlanChoice(0, 0, xc, xr))
        assert np.array_equal(got[2], ref[2]), (xc, xr)
    _lib.call("zr_plan_set", C.byref(shape), C.byref(_lib.PlanChoice(0, 0, 0, 0)))


def test_engine_plan_file_round_trip(tmp_path):
    """Engine.plan measures a new shape once and saves it; a fresh engine
    state installs the saved choice without measuring."""
    from zorro_gb300.engine import Engine
    eng = Engine.get(0)
    key = (256, 256, 128, 128, 16)
    eng._planned.discard(key)
    name, picked = eng.plan(*key, effort="FFTW_MEASURE", cache_dir=str(tmp_path))
    saved = json.load(open(tmp_path / "zorro_gb300_plans.json"))
    assert saved[name]["choice"] == picked
    eng._planned.discard(key)
    shape = _shape((256, 256), (128, 128), 16)
    _lib.call("zr_plan_set", C.byref(shape), C.byref(_lib.PlanChoice(0, 0, 0, 0)))
    name2, picked2 = eng.plan(*key, effort="FFTW_MEASURE", cache_dir=str(tmp_path))
    assert (name2, picked2) == (name, picked)
    got = _lib.PlanChoice()
    _lib.call("zr_plan_get", C.byref(shape), C.byref(got))
    assert [got.fwd_rows, got.fwd_cols, got.xc_cols, got.xc_rows] == picked
    assert eng.plan(*key, effort="FFTW_MEASURE", cache_dir=str(tmp_path)) is None  # planned already
