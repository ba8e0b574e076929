"""Host setup of the well-balanced mode against the reference (CPU): the
equilibrium arrays that SDADER_Simulator.init_equilibrium_state builds and
uploads match the ones the reference's init_equilibrium_state made for the
golden cases (src/sdader_simulator.py:436-481)."""
import platform

import numpy as np
import pytest

from golden_cases import DIMS, WB_KEYS, case_names, golden_operators, load, make_ic
from spd_gb300 import simulator as sim_mod

EXACT = platform.machine() == "x86_64"


class FakeContext:
    """Records uploads; the device is never touched."""

    def __init__(self):
        self.uploads = {}
        self.dt = 0.0

    def upload(self, name, arr):
        self.uploads[name] = np.array(arr, copy=True)

    def set_dt(self, dt):
        self.dt = dt

    def get_dt(self):
        return self.dt


def wb_cases():
    return [n for n in case_names() if load(n)[1].get("WB", False)]


def build_host_only(monkeypatch, kw, meta, data):
    monkeypatch.setattr(sim_mod.SD_Simulator, "_create_context",
                        lambda self: setattr(self, "_ctx", FakeContext()))
    monkeypatch.setattr(sim_mod.SD_Simulator, "compute_dt", lambda self: None)
    return sim_mod.SDADER_Simulator(init_fct=make_ic(meta["ic"]), operators=golden_operators(data),
                                    verbose=False, **kw)


@pytest.mark.parametrize("name", wb_cases())
def test_equilibrium_arrays_match_reference(monkeypatch, name):
    data, kw, meta = load(name)
    s = build_host_only(monkeypatch, kw, meta, data)
    ndim = s.ndim
    checked = 0
    for key in WB_KEYS:
        for field in (key, *(f"{key}_{d}" for d in DIMS[:ndim])):
            if field not in data:
                continue
            got = s._ctx.uploads[field]
            ref = data[field]
            assert got.shape == ref.shape, field
            if EXACT:
                assert np.array_equal(got, ref), field
            else:
                np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15, err_msg=field)
            assert np.array_equal(getattr(s.dm, field), got), field
            checked += 1
    assert checked == 2 + 2 * ndim + (2 * ndim + 1 if s.update == "FV" else 0)


def test_eq_fv_fb_is_refused_only_without_wb(monkeypatch):
    name = next(n for n in wb_cases() if load(n)[1].get("update") == "FV" and load(n)[1].get("FB"))
    data, kw, meta = load(name)
    assert any("eq" in sides for sides in kw["BC"])
    build_host_only(monkeypatch, kw, meta, data)  # WB=True builds
    kw = dict(kw, WB=False)
    kw.pop("eq_fct", None)
    with pytest.raises(NotImplementedError, match="WB=False"):
        build_host_only(monkeypatch, kw, meta, data)


def test_threaded_equilibrium_sampling_is_bitwise(monkeypatch):
    """Grids of more than 2^15 elements (ghosts included) sample the
    equilibrium on host thread slabs: the arrays equal the one-thread ones
    bit for bit."""
    import os
    from spd_gb300 import initial_conditions as ics
    eq = ics.gravity_column(amp=0.0)
    kw = dict(p=1, N=(182, 182), eq_fct=eq, WB=True, potential=True, update="FV", FB=True,
              BC=(("periodic", "periodic"), ("eq", "eq")))
    monkeypatch.setattr(sim_mod.SD_Simulator, "_create_context", lambda self: setattr(self, "_ctx", FakeContext()))
    monkeypatch.setattr(sim_mod.SD_Simulator, "compute_dt", lambda self: None)
    monkeypatch.setattr(os, "cpu_count", lambda: 4)
    many = sim_mod.SDADER_Simulator(init_fct=eq, verbose=False, **kw)._ctx.uploads
    monkeypatch.setattr(os, "cpu_count", lambda: 1)
    one = sim_mod.SDADER_Simulator(init_fct=eq, verbose=False, **kw)._ctx.uploads
    names = [k for k in many if "_eq_" in k]
    assert len(names) == 2 + 2 * 2 + 2 * 2 + 1
    for k in names:
        assert np.array_equal(many[k], one[k]), k
