"""ctypes binding of the C ABI in include/spd_gb300.h.

The shared library ``libspd_gb300.so`` is built in-tree next to this file
(``spd_gb300.build.build()``).  There is no CPU fallback: loading fails
loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libspd_gb300.so")
# the opt-in build with fused multiply-adds (results differ from the
# reference's in the last bits; see spd_gb300.build)
LIB_PATH_FMA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libspd_gb300_fma.so")

SPD_OK, SPD_ERR_ARG, SPD_ERR_CUDA, SPD_ERR_NONFINITE = 0, 1, 2, 3
RIEMANN = {"llf": 0, "hllc": 1, "lhllc": 2}
LIMITER = {"minmod": 0, "moncen": 1}
UPDATE = {"SD": 0, "FV": 1}
BCKIND = {"periodic": 0, "reflective": 1, "gradfree": 2, "ic": 3, "eq": 4, "pressure": 5}
FIELD = {
    "U_sp": 0, "U_cv": 1, "W_cv": 2, "troubles": 3, "theta": 4,
    "affected_faces_x": 5, "affected_faces_y": 6, "affected_faces_z": 7,
    "BC_fp_x": 8, "BC_fp_y": 9, "BC_fp_z": 10,
    "BC_fv_x": 11, "BC_fv_y": 12, "BC_fv_z": 13, "U_sp_adj": 14,
    "F_faces_x": 15, "F_faces_y": 16, "F_faces_z": 17,
    "grad_phi_sp": 18, "grad_phi_cv": 19,
    "U_eq_sp": 20, "U_eq_cv": 21, "M_eq_fp_x": 22, "M_eq_fp_y": 23, "M_eq_fp_z": 24,
    "F_eq_fp_x": 25, "F_eq_fp_y": 26, "F_eq_fp_z": 27, "M_eq_faces_x": 28, "M_eq_faces_y": 29,
    "M_eq_faces_z": 30, "F_eq_faces_x": 31, "F_eq_faces_y": 32, "F_eq_faces_z": 33, "M_eq_fv": 34,
}

# every entry point declared in include/spd_gb300.h
EXPORTS = (
    "spd_create", "spd_upload", "spd_download", "spd_compute_dt", "spd_set_dt",
    "spd_get_dt", "spd_perform_update", "spd_step", "spd_end_sim",
    "spd_synchronize", "spd_destroy", "spd_last_error", "spd_version",
    "spd_set_stream", "spd_profile", "spd_profile_report", "spd_launch_count",
    "spd_cfl_dt_noalloc", "spd_ensemble_create", "spd_ensemble_create_packed", "spd_ensemble_graph_nodes",
    "spd_ensemble_step",
    "spd_ensemble_synchronize", "spd_ensemble_time", "spd_ensemble_set_time", "spd_ensemble_destroy", "spd_ensemble_last_error",
    "spd_set_cells_per_block", "spd_get_cells_per_block",
    "spd_adjoint_enable", "spd_adjoint_depth", "spd_record_step", "spd_vjp_step",
    "spd_tape_enable", "spd_tape_step",
)


class spd_config(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int),
        ("N", ctypes.c_int * 3),
        ("p", ctypes.c_int),
        ("m", ctypes.c_int),
        ("lim", (ctypes.c_double * 2) * 3),
        ("gamma", ctypes.c_double),
        ("cfl_coeff", ctypes.c_double),
        ("min_c2", ctypes.c_double),
        ("riemann_solver_sd", ctypes.c_int),
        ("riemann_solver_fv", ctypes.c_int),
        ("slope_limiter", ctypes.c_int),
        ("update", ctypes.c_int),
        ("FB", ctypes.c_int),
        ("tolerance", ctypes.c_double),
        ("SED", ctypes.c_int),
        ("NAD_delta", ctypes.c_int),
        ("PAD", ctypes.c_int),
        ("blending", ctypes.c_int),
        ("min_rho", ctypes.c_double),
        ("max_rho", ctypes.c_double),
        ("min_P", ctypes.c_double),
        ("godunov", ctypes.c_int),
        ("BC", (ctypes.c_int * 2) * 3),
        ("viscosity", ctypes.c_int),
        ("nu", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("potential", ctypes.c_int),
        ("isothermal", ctypes.c_int),
        ("WB", ctypes.c_int),
    ]


_dp = ctypes.POINTER(ctypes.c_double)


class spd_operators(ctypes.Structure):
    _fields_ = [
        ("sp_to_fp", _dp),
        ("dfp_to_sp", _dp),
        ("sp_to_cv", _dp),
        ("cv_to_sp", _dp),
        ("invader", _dp),
        ("w_tp", _dp),
        ("faces", _dp * 3),
    ]


class SpdError(RuntimeError):
    """Error reported by the CUDA library."""


_LIBS = {}


def load(variant: str = "ieee"):
    """Load a library variant once ("ieee": the product, bit-identical to
    the reference; "fma": fused multiply-adds) and declare the signatures."""
    if variant in _LIBS:
        return _LIBS[variant]
    path = {"ieee": LIB_PATH, "fma": LIB_PATH_FMA}[variant]
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with spd_gb300.build.build() "
            "(spd_gb300 has no CPU fallback)")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    lib.spd_create.argtypes = [ctypes.POINTER(spd_config), ctypes.POINTER(spd_operators), ctypes.POINTER(vp)]
    lib.spd_upload.argtypes = [vp, ctypes.c_int, _dp, ctypes.c_size_t]
    lib.spd_download.argtypes = [vp, ctypes.c_int, _dp, ctypes.c_size_t]
    lib.spd_compute_dt.argtypes = [vp, _dp]
    lib.spd_set_dt.argtypes = [vp, ctypes.c_double]
    lib.spd_get_dt.argtypes = [vp, _dp]
    lib.spd_perform_update.argtypes = [vp, _dp]
    lib.spd_step.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_int)]
    lib.spd_end_sim.argtypes = [vp]
    lib.spd_synchronize.argtypes = [vp]
    lib.spd_destroy.argtypes = [vp]
    lib.spd_last_error.argtypes = [vp]
    lib.spd_set_stream.argtypes = [vp, vp]
    lib.spd_profile.argtypes = [vp, ctypes.c_int]
    lib.spd_profile_report.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.spd_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    lib.spd_adjoint_enable.argtypes = [vp, ctypes.c_int]
    lib.spd_adjoint_depth.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    lib.spd_record_step.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    lib.spd_vjp_step.argtypes = [vp, ctypes.c_int]
    lib.spd_tape_enable.argtypes = [vp, ctypes.c_int]
    lib.spd_tape_step.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.spd_last_error.restype = ctypes.c_char_p
    lib.spd_version.restype = ctypes.c_char_p
    for name in EXPORTS:
        getattr(lib, name).restype = getattr(lib, name).restype or ctypes.c_int
    lib.spd_last_error.restype = ctypes.c_char_p
    lib.spd_version.restype = ctypes.c_char_p
    lib.spd_variant = variant
    _LIBS[variant] = lib
    return lib


def as_ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class Context:
    """Owns one spd_ctx (one CUDA stream, device state of one simulation)."""

    def __init__(self, cfg: spd_config, mats: dict, faces: list, variant: str = "ieee"):
        self.lib = load(variant)
        self.variant = variant
        self._keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in mats.items()}
        self._faces = [np.ascontiguousarray(f, dtype=np.float64) for f in faces]
        ops = spd_operators()
        for k in ("sp_to_fp", "dfp_to_sp", "sp_to_cv", "cv_to_sp", "invader", "w_tp"):
            setattr(ops, k, as_ptr(self._keep[k]))
        for d in range(3):
            ops.faces[d] = as_ptr(self._faces[d]) if d < len(self._faces) else None
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self.lib.spd_create(ctypes.byref(cfg), ctypes.byref(ops), ctypes.byref(h))
        if rc != SPD_OK:
            raise SpdError(f"spd_create failed with status {rc}")
        self.h = h

    def check(self, rc, what):
        if rc != SPD_OK:
            msg = self.lib.spd_last_error(self.h)
            raise SpdError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def upload(self, field: str, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self.check(self.lib.spd_upload(self.h, FIELD[field], as_ptr(a), a.size), f"upload {field}")

    def download(self, field: str, shape) -> np.ndarray:
        out = np.empty(shape, dtype=np.float64)
        self.check(self.lib.spd_download(self.h, FIELD[field], as_ptr(out), out.size), f"download {field}")
        return out

    def upload_ptr(self, field: str, ptr: int, count: int):
        """Upload from a host or device address (count doubles, reference layout)."""
        self.check(self.lib.spd_upload(self.h, FIELD[field], ctypes.cast(ctypes.c_void_p(ptr), _dp), int(count)),
                   f"upload {field}")

    def download_ptr(self, field: str, ptr: int, count: int):
        """Download into a host or device address (count doubles, reference layout)."""
        self.check(self.lib.spd_download(self.h, FIELD[field], ctypes.cast(ctypes.c_void_p(ptr), _dp), int(count)),
                   f"download {field}")

    def adjoint_enable(self, depth: int):
        self.check(self.lib.spd_adjoint_enable(self.h, int(depth)), "adjoint_enable")

    def adjoint_depth(self) -> int:
        n = ctypes.c_int()
        self.check(self.lib.spd_adjoint_depth(self.h, ctypes.byref(n)), "adjoint_depth")
        return n.value

    def record_step(self, slot: int, dt: float):
        self.check(self.lib.spd_record_step(self.h, int(slot), float(dt)), "record_step")

    def vjp_step(self, slot: int):
        self.check(self.lib.spd_vjp_step(self.h, int(slot)), "vjp_step")

    def tape_enable(self, nsteps: int):
        self.check(self.lib.spd_tape_enable(self.h, int(nsteps)), "tape_enable")

    def tape_step(self, step: int, dt: float, mode: int):
        """mode 1: step and record its decisions; mode 2: step replaying them."""
        self.check(self.lib.spd_tape_step(self.h, int(step), float(dt), int(mode)), "tape_step")

    def compute_dt(self) -> float:
        dt = ctypes.c_double()
        self.check(self.lib.spd_compute_dt(self.h, ctypes.byref(dt)), "compute_dt")
        return dt.value

    def set_dt(self, dt: float):
        self.check(self.lib.spd_set_dt(self.h, float(dt)), "set_dt")

    def get_dt(self) -> float:
        dt = ctypes.c_double()
        self.check(self.lib.spd_get_dt(self.h, ctypes.byref(dt)), "get_dt")
        return dt.value

    def perform_update(self, time: float) -> float:
        t = ctypes.c_double(time)
        self.check(self.lib.spd_perform_update(self.h, ctypes.byref(t)), "perform_update")
        return t.value

    def step(self, nsteps: int, t_end: float, mode: int, time: float):
        """Returns (time, steps done, True when a dt was not finite)."""
        t = ctypes.c_double(time)
        done = ctypes.c_int(0)
        rc = self.lib.spd_step(self.h, int(nsteps), float(t_end), int(mode), ctypes.byref(t), ctypes.byref(done))
        if rc != SPD_ERR_NONFINITE:
            self.check(rc, "step")
        return t.value, done.value, rc == SPD_ERR_NONFINITE

    def end_sim(self):
        self.check(self.lib.spd_end_sim(self.h), "end_sim")

    def synchronize(self):
        self.check(self.lib.spd_synchronize(self.h), "synchronize")

    def set_stream(self, stream_handle: int | None):
        self.check(self.lib.spd_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)), "set_stream")

    def profile(self, enable: bool):
        self.check(self.lib.spd_profile(self.h, int(bool(enable))), "profile")

    def profile_report(self) -> dict:
        """{kernel: (launches, total_ms)} recorded since the last report."""
        buf = ctypes.create_string_buffer(1 << 16)
        self.check(self.lib.spd_profile_report(self.h, buf, len(buf)), "profile_report")
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        self.check(self.lib.spd_launch_count(self.h, ctypes.byref(n)), "launch_count")
        return n.value

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.spd_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
