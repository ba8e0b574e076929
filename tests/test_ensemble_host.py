"""Host logic of SDADER_Ensemble on a stand-in for the C library (CPU):
the choice between the packed and the stream form, the autotuner's
candidates and pick, the bookkeeping of each instance's time and step count
around a launch, and the error raised by a failed create."""
import ctypes
import types

import pytest

from spd_gb300 import _lib
from spd_gb300 import ensemble as ens_mod


class FakeLib:
    """The spd_ensemble_* entry points as Python callables: every launch
    adds 0.25 to each instance's device time; probe launches of the
    candidate (packed, cells per block 32) are the fastest."""

    def __init__(self, fail_create=False, fail_packed=False):
        self.fail_create = fail_create
        self.fail_packed = fail_packed
        self.created = []
        self.times = {}
        self.cpb = {}
        self.current = None
        self.last_err = b""

    def _declare(self):
        return None

    # creation
    def spd_ensemble_create_packed(self, arr, n, spl, ref):
        return self._create("packed", None, n, spl, ref)

    def spd_ensemble_create(self, arr, n, nstreams, spl, ref):
        return self._create("streams", nstreams, n, spl, ref)

    def _create(self, form, nstreams, n, spl, ref):
        if self.fail_create or (self.fail_packed and form == "packed"):
            self.last_err = b"instances differ at launch 3 (k_nad): options, degree or cells per block"
            return 1
        handle = len(self.created) + 1
        self.created.append((form, nstreams, n, spl))
        self.current = (form, nstreams)
        ref._obj.value = handle
        return 0

    def spd_ensemble_last_error(self, h):
        return self.last_err

    def spd_ensemble_graph_nodes(self, h, ref):
        ref._obj.value = 131
        return 0

    def spd_ensemble_destroy(self, h):
        return 0

    def spd_ensemble_set_time(self, h, i, t):
        self.times[i] = t
        return 0

    def spd_ensemble_time(self, h, i, ref):
        ref._obj.value = self.times[i]
        return 0

    def spd_ensemble_step(self, h, launches):
        form, ns = self.current
        cpb = next(iter(self.cpb.values()), 32)
        self.delay = 0.0 if (form == "packed" and cpb == 32) else 0.002
        for i in self.times:
            self.times[i] += 0.25 * launches
        import time
        time.sleep(self.delay * launches)
        return 0

    def spd_ensemble_synchronize(self, h):
        return 0

    def spd_get_cells_per_block(self, h, cref, mref):
        cref._obj.value = self.cpb.get(h.value if hasattr(h, "value") else h, 32)
        mref._obj.value = 64
        return 0

    def spd_set_cells_per_block(self, h, cpb):
        self.cpb[h.value if hasattr(h, "value") else h] = cpb
        return 0


def _sims(n):
    return [types.SimpleNamespace(_ctx=types.SimpleNamespace(h=ctypes.c_void_p(100 + i)), time=0.5 * i, n_step=3)
            for i in range(n)]


@pytest.fixture
def fake(monkeypatch):
    lib = FakeLib()
    monkeypatch.setattr(_lib, "load", lambda *a: lib)
    monkeypatch.setattr(ens_mod.SDADER_Ensemble, "_declare", lambda self: None)
    return lib


def test_default_is_packed_and_steps_update_time(fake):
    sims = _sims(3)
    e = ens_mod.SDADER_Ensemble(sims, steps_per_launch=2)
    assert fake.created[-1][0] == "packed" and fake.created[-1][2] == 3
    e.perform_iterations(4)  # 2 launches
    assert [s.time for s in sims] == [0.5, 1.0, 1.5]  # 0.5 * i + 2 launches x 0.25
    assert [s.n_step for s in sims] == [7, 7, 7]
    with pytest.raises(ValueError):
        e.perform_iterations(3)
    assert e.graph_nodes() == 131


def test_stream_form_on_request(fake):
    ens_mod.SDADER_Ensemble(_sims(2), nstreams=4, packed=False)
    assert fake.created[-1][:2] == ("streams", 4)


def test_autotune_tries_every_candidate_and_keeps_the_fastest(fake):
    sims = _sims(2)
    e = ens_mod.SDADER_Ensemble(sims)
    tuning = e.autotune(streams=(1, 4), cpbs=(16, 32), probe_launches=1)
    # 2 cells-per-block values x (packed, 1 stream, 4 streams), each built once
    assert len(fake.created) == 1 + 6 + 1
    assert tuning["form"] == "packed" and tuning["cells_per_block"] == 32 and tuning["streams"] is None
    assert len(tuning["candidates"]) == 6
    assert fake.created[-1][0] == "packed"  # rebuilt with the choice
    assert all(s.n_step == 3 + 6 * 2 for s in sims)  # each probe: 1 warm-up + 1 timed step


def test_autotune_skips_a_packed_form_that_cannot_be_created(monkeypatch):
    """Instances that differ in degree or options: the packed create fails,
    autotune keeps timing the stream forms and builds the fastest of them."""
    lib = FakeLib(fail_packed=True)
    monkeypatch.setattr(_lib, "load", lambda *a: lib)
    monkeypatch.setattr(ens_mod.SDADER_Ensemble, "_declare", lambda self: None)
    sims = _sims(2)
    e = ens_mod.SDADER_Ensemble(sims, packed=False, nstreams=2)
    tuning = e.autotune(streams=(1, 4), cpbs=(16, 32), probe_launches=1)
    assert tuning["form"] == "streams"
    assert len(tuning["candidates"]) == 4 and len(tuning["skipped"]) == 2
    assert all("instances differ" in v for v in tuning["skipped"].values())
    assert e._ens is not None and lib.created[-1][0] == "streams"
    e.perform_iterations(1)  # the chosen form is live


def test_autotune_with_no_buildable_candidate_restores_the_previous_form(monkeypatch):
    lib = FakeLib(fail_packed=True)
    monkeypatch.setattr(_lib, "load", lambda *a: lib)
    monkeypatch.setattr(ens_mod.SDADER_Ensemble, "_declare", lambda self: None)
    sims = _sims(2)
    e = ens_mod.SDADER_Ensemble(sims, packed=False, nstreams=3)
    with pytest.raises(_lib.SpdError, match="no candidate"):
        e.autotune(streams=(1,), cpbs=(16,), probe_launches=1, packed=(True,))
    assert lib.created[-1][:2] == ("streams", 3) and e._ens is not None
    e.perform_iterations(1)


def test_failed_create_explains_itself(monkeypatch):
    lib = FakeLib(fail_create=True)
    monkeypatch.setattr(_lib, "load", lambda *a: lib)
    monkeypatch.setattr(ens_mod.SDADER_Ensemble, "_declare", lambda self: None)
    with pytest.raises(_lib.SpdError, match="packed=False"):
        ens_mod.SDADER_Ensemble(_sims(2))
    with pytest.raises(_lib.SpdError, match="instances differ"):
        ens_mod.SDADER_Ensemble(_sims(2), packed=False)


def test_empty_ensemble_is_rejected(fake):
    with pytest.raises(ValueError):
        ens_mod.SDADER_Ensemble([])
