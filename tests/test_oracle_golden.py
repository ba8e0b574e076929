"""The oracle restatement against the reference's own outputs (CPU)."""
import numpy as np
import pytest

from golden_cases import case_names, load, oracle_from_golden, DIMS


@pytest.mark.parametrize("name", case_names())
def test_oracle_matches_reference_bitwise(name):
    data, kw, meta = load(name)
    o = oracle_from_golden(data, kw)
    dts = []
    for _ in range(meta["steps"]):
        dts.append(o.compute_dt())
        o.perform_update()
    assert np.array_equal(np.array(dts), data["dts"])
    assert o.time == float(data["time"])
    for key, val in (("U_sp", o.U_sp), ("U_cv", o.U_cv), ("W_cv", o.W_cv)):
        assert np.array_equal(val, data[key], equal_nan=True), key
    if "troubles" in data:
        assert np.array_equal(o.troubles, data["troubles"])
        assert np.array_equal(o.theta, data["theta"])
        for i in range(len(kw["N"])):
            assert np.array_equal(o.affected[i], data[f"affected_faces_{DIMS[i]}"])


def test_oracle_sees_troubles():
    """The limiter cases really exercise trouble detection."""
    data, kw, meta = load("quadrant16_p3_fvfb_hllc_gradfree")
    assert data["troubles"].sum() > 0
    assert data["theta"].max() > 1.0  # boundary contamination of theta


@pytest.mark.parametrize("name", case_names())
def test_torch_transcription_matches_reference_bitwise(name):
    """The oracle run on torch tensors (the FP64 torch transcription whose
    autograd gradient checks the CUDA adjoint) reproduces the reference's
    outputs bit for bit, like the NumPy run."""
    torch = pytest.importorskip("torch")
    data, kw, meta = load(name)
    o = oracle_from_golden({**data, "init_U_sp": torch.tensor(data["init_U_sp"])}, kw)
    for _ in range(meta["steps"]):
        o.compute_dt()
        o.perform_update()
    assert isinstance(o.U_sp, torch.Tensor)
    assert np.array_equal(o.U_sp.numpy(), data["U_sp"])
