"""Host logic of the autotuner (tfce_mediation_gb300/autotune.py) with the
device timings replaced by fixed numbers: which GLM form and tile it keeps,
which (CTA shape, P) it keeps, and that a cached choice is restored on a new
engine without timing anything.  No GPU needed."""
import pytest

from tfce_mediation_gb300 import autotune as A


class _TC:
    def __init__(self):
        self.quadratic_form = True
        self.design_block = None
        self.glm_timings = None


class _Adj:
    n_entries = 1000

    def __init__(self):
        self.shape = None

    def set_sweep_shape(self, s):
        self.shape = s

    def resident_slots(self):
        return 456


class _Eng:
    def __init__(self, k=5, qf_allowed=True):
        self.k, self.n, self.V, self.n_seg, self.C, self.signs = k, 100, 5000, 2, 4, 2
        self.precision = "bf16x3"
        self._tc = _TC()
        self.adj = _Adj()
        self._qf_allowed = qf_allowed

    def _graph_qf(self):
        return self._qf_allowed and self._tc.quadratic_form


def _glm_clock(times):
    def time_glm(eng, P):
        tc = eng._tc
        return times["qf"] if tc.quadratic_form else times[tc.design_block]
    return time_glm


def test_quadratic_form_kept_when_faster(monkeypatch):
    monkeypatch.setattr(A, "time_glm", _glm_clock({"qf": 2.0, 32: 8.0, 16: 9.0}))
    eng = _Eng()
    assert A.choose_design_block(eng, 256) == (32, True)
    assert eng._tc.quadratic_form and eng._tc.design_block == 32
    assert eng._tc.glm_timings == {"qf": 2.0, "res32": 8.0, "res16": 9.0}


def test_residual_epilogue_kept_when_faster(monkeypatch):
    monkeypatch.setattr(A, "time_glm", _glm_clock({"qf": 12.0, 32: 8.0, 16: 7.0}))
    eng = _Eng()
    assert A.choose_design_block(eng, 256) == (16, False)
    assert not eng._tc.quadratic_form


def test_only_the_forms_that_apply_are_timed(monkeypatch):
    seen = []

    def time_glm(eng, P):
        seen.append("qf" if eng._tc.quadratic_form else eng._tc.design_block)
        return 1.0
    monkeypatch.setattr(A, "time_glm", time_glm)
    # more than 5 columns: only 16-design tiles exist for the residual epilogue
    assert A.choose_design_block(_Eng(k=7), 64) == (16, True)
    assert seen == ["qf", 16]
    # an engine whose GLM cannot take the quadratic form (an output program)
    seen.clear()
    assert A.choose_design_block(_Eng(qf_allowed=False), 64) == (32, False)
    assert seen == [32, 16]


def test_choice_is_cached_and_restored(monkeypatch, tmp_path):
    monkeypatch.setattr(A, "CACHE", str(tmp_path / "autotune.json"))
    monkeypatch.setattr(A, "_key", lambda eng: "fake-gpu|problem")
    monkeypatch.setattr(A, "time_glm", _glm_clock({"qf": 2.0, 32: 8.0, 16: 9.0}))
    rates = {(3, 256): 5.0, (2, 256): 4.0}

    def time_batch(eng, P):
        return P / rates.get((eng.adj.shape, P), 1.0)
    monkeypatch.setattr(A, "time_batch", time_batch)
    eng = _Eng()
    assert A.choose_batch(eng, max_p=256) == 256
    assert eng.adj.shape == 3 and eng._tc.quadratic_form

    def no_timing(*_):
        raise AssertionError("a cached choice is not timed again")
    monkeypatch.setattr(A, "time_glm", no_timing)
    monkeypatch.setattr(A, "time_batch", no_timing)
    again = _Eng()
    again._tc.quadratic_form = False
    assert A.choose_batch(again, max_p=256) == 256
    assert again.adj.shape == 3 and again._tc.quadratic_form and again._tc.design_block == 32
    assert again._tc.glm_timings == {"qf": 2.0, "res32": 8.0, "res16": 9.0}


@pytest.mark.parametrize("ctas", [456, 304])
def test_candidates_fill_whole_waves(ctas):
    eng = _Eng()
    eng.adj.resident_slots = lambda: ctas
    per_perm = eng.C * eng.signs * eng.n_seg
    for P in A.candidates(eng, 256):
        assert 4 <= P <= 256
        assert P in (16, 32, 64, 128, 256) or (P * per_perm) % ctas == 0
