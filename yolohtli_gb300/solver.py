"""The solver handle (yh_create ... yh_destroy) as a Python class.

Host arrays are numpy FP32 (flat nx*ny, row-major idx = i + nx*j). The handle
owns its device buffers; `run` replays captured CUDA graphs.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from ._loader import load
from .ops import check


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def _fptr(x):
    return None if x is None else x.ctypes.data_as(C.c_void_p)


class Monodomain:
    """One grid of the 2D monodomain model on the GPU."""

    def __init__(self, p, model=A.YH_MODEL_FK3V, fk=None, solid=None,
                 stream=None):
        self.lib = load()
        self.p = p.copy()
        self.model = model
        self.nf = A.NFIELDS[model]
        self.fk = fk if fk is not None else A.fk_defaults()
        self._solid = None
        if solid is not None:
            self._solid = np.ascontiguousarray(solid, dtype=np.uint8)
            self.p.solidSwitch = True
        h = C.c_void_p()
        check("yh_create", self.lib.yh_create(
            C.byref(self.p), model, C.byref(self.fk),
            None if self._solid is None else self._solid.ctypes.data_as(C.c_void_p),
            C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    @property
    def has_mask(self):
        return self._solid is not None

    @property
    def n(self):
        return self.p.nx * self.p.ny

    def close(self):
        if getattr(self, "h", None):
            self.lib.yh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, u, v, w=None):
        arrs = [_f32(u), _f32(v), None if w is None else _f32(w)]
        self._keep = arrs
        check("yh_set_state", self.lib.yh_set_state(
            self.h, *[_fptr(a) for a in arrs]))

    def get_state(self):
        out = [np.empty(self.n, np.float32) for _ in range(self.nf)]
        ptrs = [_fptr(a) for a in out] + [None] * (3 - self.nf)
        check("yh_get_state", self.lib.yh_get_state(self.h, *ptrs))
        return out

    def state_device(self):
        f = A.Fields()
        check("yh_state_device", self.lib.yh_state_device(self.h, C.byref(f)))
        return f

    def set_time_block(self, k):
        check("yh_set_time_block", self.lib.yh_set_time_block(self.h, int(k)))

    def time_block(self):
        k = C.c_int()
        check("yh_get_time_block", self.lib.yh_get_time_block(self.h, C.byref(k)))
        return k.value

    def set_engine(self, engine, steps_per_launch=1):
        check("yh_set_engine", self.lib.yh_set_engine(
            self.h, int(engine), int(steps_per_launch)))

    def engine(self):
        e, k = C.c_int(), C.c_int()
        check("yh_get_engine", self.lib.yh_get_engine(self.h, C.byref(e), C.byref(k)))
        return e.value, k.value

    def autotune(self, probe_steps=256):
        """Picks the fastest engine/depth on the current state (restored);
        returns (engine, steps_per_launch)."""
        e, k = C.c_int(), C.c_int()
        check("yh_autotune", self.lib.yh_autotune(
            self.h, int(probe_steps), C.byref(e), C.byref(k)))
        return e.value, k.value

    def run(self, nsteps, stims=()):
        arr = (A.Stim * max(1, len(stims)))(*stims)
        check("yh_run", self.lib.yh_run(self.h, int(nsteps), arr, len(stims)))

    def synchronize(self):
        check("yh_synchronize", self.lib.yh_synchronize(self.h))

    def step_count(self):
        s = C.c_int()
        check("yh_get_step", self.lib.yh_get_step(self.h, C.byref(s)))
        return s.value

    def set_step(self, step):
        check("yh_set_step", self.lib.yh_set_step(self.h, int(step)))

    def launch_count(self):
        n = C.c_longlong()
        check("yh_get_launch_count",
              self.lib.yh_get_launch_count(self.h, C.byref(n)))
        return n.value

    def check_finite(self):
        """The number of NaN or Inf values in the state (0: all finite)."""
        n = C.c_longlong()
        st = self.lib.yh_check_finite(self.h, C.byref(n))
        if st not in (A.YH_OK, A.YH_ENONFINITE):
            check("yh_check_finite", st)
        return n.value

    def save_checkpoint(self, path):
        """State, step count, parameters and mask in this library's binary
        checkpoint file (yolohtli_gb300.checkpoint)."""
        check("yh_save_checkpoint",
              self.lib.yh_save_checkpoint(self.h, str(path).encode()))

    def load_checkpoint(self, path):
        """Restores state and step count from a checkpoint of the same
        problem (grid, model, step coefficients, FK3V parameters, mask)."""
        check("yh_load_checkpoint",
              self.lib.yh_load_checkpoint(self.h, str(path).encode()))

    def run_checked(self, nsteps, stims=(), every=1000):
        """run() in segments of `every` steps, each followed by
        check_finite(). The state and step count after the last finite
        segment are kept on the host. When a segment ends with a NaN or Inf
        in the state, the handle is rolled back to them and YolohtliError
        (YH_ENONFINITE) is raised. The explicit step is deterministic, so
        running the same segment again fails again: the caller changes dt
        or the state first. Returns the number of segments run."""
        every = max(1, int(every))
        good = (self.get_state(), self.step_count())
        left, segments = int(nsteps), 0
        while left > 0:
            m = min(every, left)
            self.run(m, stims)
            segments += 1
            if self.check_finite():
                state, step = good
                self.set_state(*state)
                self.set_step(step)
                self.synchronize()
                check("yh_check_finite", A.YH_ENONFINITE)
            left -= m
            if left > 0:
                good = (self.get_state(), self.step_count())
        return segments

    def track_tips(self):
        check("yh_track_tips", self.lib.yh_track_tips(self.h))

    def get_tips(self, capacity=1 << 16):
        buf = (A.Tip * capacity)()
        n = C.c_int()
        st = self.lib.yh_get_tips(self.h, buf, capacity, C.byref(n))
        if st not in (A.YH_OK, A.YH_EOVERFLOW):
            check("yh_get_tips", st)
        m = min(n.value, capacity)
        return np.array([[buf[k].x, buf[k].y, buf[k].vx, buf[k].vy, buf[k].t]
                         for k in range(m)], np.float32).reshape(m, 5)

    def save_raw_data(self, path):
        """The state as the reference's raw_data.dat ("u v" per cell)."""
        from . import refio
        u, v = self.get_state()[:2]
        refio.write_raw_data(path, self.p, u, v)

    def save_param_csv(self, path, ic_path=None, results_path=None):
        """The parameters as the reference's dataparamcsv.csv."""
        from . import refio
        refio.write_param_csv(path, self.p, ic_path, results_path)

    def sr_begin(self, template_mode=A.YH_TEMPLATE_CURRENT, template=None):
        t = [None, None, None]
        if template is not None:
            t = [_f32(x) for x in template] + [None] * (3 - len(template))
        self._tkeep = t
        check("yh_sr_begin", self.lib.yh_sr_begin(
            self.h, template_mode, *[_fptr(a) for a in t]))

    def sr_step(self, nsteps=1):
        check("yh_sr_step", self.lib.yh_sr_step(self.h, int(nsteps)))

    def sr_enqueue(self, nsteps=1):
        """sr_step without waiting: the steps are enqueued on the handle's
        stream; sr_status() waits and reports a singular solve."""
        check("yh_sr_enqueue", self.lib.yh_sr_enqueue(self.h, int(nsteps)))

    def sr_status(self):
        check("yh_sr_status", self.lib.yh_sr_status(self.h))

    def get_sym(self):
        s = A.SymState()
        check("yh_get_sym", self.lib.yh_get_sym(self.h, C.byref(s)))
        return s
