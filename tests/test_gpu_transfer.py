"""Uploads and downloads of the state through the C ABI from pinned host
buffers (read and written by the layout kernel over the host link) give
the same arrays as those from pageable buffers (device staging copy), for
the solution-point and the subcell layouts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(shape):
    import torch
    return torch.empty(int(np.prod(shape)), dtype=torch.float64, pin_memory=True).numpy().reshape(shape)


@pytest.mark.parametrize("N,p", [((7, 5), 3), ((4, 3, 5), 2), ((9,), 4)])
def test_pinned_and_pageable_transfers_agree(N, p):
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(p=p, N=N, update="FV", FB=True, verbose=False)
    rng = np.random.default_rng(7)
    for name in ("U_sp", "U_cv", "W_cv"):
        shape = s._shape_of(name)
        ref = rng.standard_normal(shape)
        pin = _pinned(shape)
        pin[...] = ref
        s._ctx.upload(name, pin)                      # pinned in
        got = s._ctx.download(name, shape)            # pageable out
        assert np.array_equal(got, ref), name
        s._ctx.upload(name, ref.copy())               # pageable in
        out = _pinned(shape)
        out[...] = np.nan
        s._ctx.download_ptr(name, out.ctypes.data, out.size)   # pinned out
        assert np.array_equal(out, ref), name
    s.close()
