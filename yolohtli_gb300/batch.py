"""The batched solver (yh_batch_* in include/yolohtli.h) as a Python class.

Many independent FK3V grids, each with its own size, parameters, hole mask
and stimulus events, advanced together: one kernel launch per step for each
group of instances that fits in the L2, the groups on several streams, or
one persistent launch per run (the wavefront engine, set_wave). Host
arrays are numpy FP32, flat nx*ny, row-major.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from ._loader import load
from .ops import check


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


class Batch:
    """params, fks: one ParamVar / FKParams per instance; masks: one uint8
    array (nonzero = tissue) or None per instance."""

    def __init__(self, params, fks, masks=None, stream=None):
        self.lib = load()
        n = len(params)
        if masks is None:
            masks = [None] * n
        if not (len(fks) == n == len(masks)):
            raise ValueError("params, fks and masks differ in length")
        self.params = (A.ParamVar * n)(*[p.copy() for p in params])
        self.fks = (A.FKParams * n)(*fks)
        self._masks = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8)
                       for m in masks]
        for k, m in enumerate(self._masks):
            self.params[k].solidSwitch = m is not None
        mp = (C.c_void_p * n)(*[None if m is None else m.ctypes.data
                                for m in self._masks])
        h = C.c_void_p()
        check("yh_batch_create", self.lib.yh_batch_create(
            n, self.params, self.fks, mp,
            C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h
        self.count = n

    def shape(self, k):
        return self.params[k].ny, self.params[k].nx

    def close(self):
        if getattr(self, "h", None):
            self.lib.yh_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, k, u, v, w):
        u, v, w = _f32(u), _f32(v), _f32(w)
        check("yh_batch_set_state", self.lib.yh_batch_set_state(
            self.h, k, u.ctypes.data, v.ctypes.data, w.ctypes.data))

    def get_state(self, k):
        ny, nx = self.shape(k)
        out = [np.empty(nx * ny, np.float32) for _ in range(3)]
        check("yh_batch_get_state", self.lib.yh_batch_get_state(
            self.h, k, *[o.ctypes.data for o in out]))
        return out

    def state_device(self, k):
        f = A.Fields()
        check("yh_batch_state_device", self.lib.yh_batch_state_device(
            self.h, k, C.byref(f)))
        return f

    def run(self, nsteps, stims=()):
        """stims: (instance, Stim) pairs."""
        arr = (A.BatchStim * max(1, len(stims)))()
        for q, (k, s) in enumerate(stims):
            arr[q].instance = k
            arr[q].s = s
        check("yh_batch_run", self.lib.yh_batch_run(
            self.h, int(nsteps), arr, len(stims)))

    def run_host(self, nsteps, states_in=None, states_out=None, stims=()):
        """run() with the states in host memory: states_in[k] = (u, v, w)
        arrays (or None) copied into instance k before its first step,
        states_out[k] = (u, v, w) float32 arrays (or None) filled with its
        result; under the per-instance schedule every instance's copies run
        on its own stream beside the others' steps (pinned arrays, e.g.
        torch's pin_memory(), let them overlap). Returns when the outputs
        are written."""
        n = self.count
        arr = (A.BatchStim * max(1, len(stims)))()
        for q, (k, s) in enumerate(stims):
            arr[q].instance = k
            arr[q].s = s

        def table(states, f):
            t = (C.c_void_p * n)()
            if states is not None:
                for k in range(n):
                    if states[k] is not None and states[k][f] is not None:
                        x = states[k][f]
                        t[k] = x.data_ptr() if hasattr(x, "data_ptr") else x.ctypes.data
            return t
        ins = [table(states_in, f) for f in range(3)]
        outs = [table(states_out, f) for f in range(3)]
        check("yh_batch_run_host", self.lib.yh_batch_run_host(
            self.h, int(nsteps), arr, len(stims), *ins, *outs))

    def set_schedule(self, group_cells, streams):
        """Groups of about group_cells cells on `streams` internal streams
        (group_cells 0: every instance its own sequence of single-grid step
        launches, the instances spread over the streams)."""
        check("yh_batch_set_schedule", self.lib.yh_batch_set_schedule(
            self.h, int(group_cells), int(streams)))

    def autotune(self, probe_steps=256):
        """Times the schedules on the current state (restored), keeps the
        fastest; returns (group_cells, streams, steps per launch):
        (0, streams, 1) for one launch sequence per instance, (0, CTAs per
        instance, 0) for the wavefront engine."""
        g, q, d = C.c_longlong(), C.c_int(), C.c_int()
        check("yh_batch_autotune", self.lib.yh_batch_autotune(
            self.h, int(probe_steps), C.byref(g), C.byref(q), C.byref(d)))
        return g.value, q.value, d.value

    def set_depth(self, depth):
        """Steps per launch: 1, or 2 (TMA-staged 64 x 16 tiles)."""
        check("yh_batch_set_depth", self.lib.yh_batch_set_depth(self.h, int(depth)))

    def set_wave(self, cluster, max_levels=0):
        """The wavefront engine (one persistent launch per run segment) with
        `cluster` CTAs per instance (1, 2 or 4; 0: grouped launches) and at
        most max_levels steps per pass (0: as many as the rings allow)."""
        check("yh_batch_set_wave", self.lib.yh_batch_set_wave(
            self.h, int(cluster), int(max_levels)))

    def wave(self):
        """(CTAs per instance or 0, levels cap, clusters of the launch)."""
        c, k, n = C.c_int(), C.c_int(), C.c_int()
        check("yh_batch_get_wave", self.lib.yh_batch_get_wave(
            self.h, C.byref(c), C.byref(k), C.byref(n)))
        return c.value, k.value, n.value

    def synchronize(self):
        check("yh_batch_synchronize", self.lib.yh_batch_synchronize(self.h))

    def step_count(self):
        s = C.c_int()
        check("yh_batch_get_step", self.lib.yh_batch_get_step(self.h, C.byref(s)))
        return s.value

    def set_step(self, step):
        check("yh_batch_set_step", self.lib.yh_batch_set_step(self.h, int(step)))

    @staticmethod
    def checkpoint_path(directory, k):
        import os
        return os.path.join(str(directory), "instance_%04d.yhck" % k)

    def save_checkpoint(self, directory):
        """One checkpoint file per instance (yolohtli_gb300.checkpoint), all
        at the batch's step, in `directory`. The files go to a fresh
        directory `directory`.tmp first; only when all of them are written
        does it replace `directory` (the old one is moved to `directory`.old
        and removed after the swap). An interrupted save leaves the previous
        checkpoint in `directory`, or, inside the swap, in `directory`.old,
        which load_checkpoint falls back to."""
        import os
        import shutil
        from . import checkpoint as ck
        d = os.path.normpath(str(directory))
        tmp, old = d + ".tmp", d + ".old"
        shutil.rmtree(tmp, ignore_errors=True)
        os.makedirs(tmp)
        step = self.step_count()
        for k in range(self.count):
            ck.write(self.checkpoint_path(tmp, k), self.params[k],
                     A.YH_MODEL_FK3V, self.fks[k], step, *self.get_state(k),
                     mask=self._masks[k])
        if os.path.exists(d):
            shutil.rmtree(old, ignore_errors=True)
            os.rename(d, old)
        os.rename(tmp, d)
        shutil.rmtree(old, ignore_errors=True)

    def load_checkpoint(self, directory):
        """Restores every instance's state and the step from the files of
        save_checkpoint. Every file is read and checked first: a corrupt
        file raises YH_ECORRUPT, another problem (an instance's grid, step
        coefficients, FK3V parameters or mask) or files at different steps
        raise YH_EINVAL, and the batch is left as it was."""
        import os
        from . import checkpoint as ck
        d = os.path.normpath(str(directory))
        if not os.path.exists(d) and os.path.exists(d + ".old"):
            d = d + ".old"  # a save interrupted inside its directory swap
        got = [ck.read(self.checkpoint_path(d, k)) for k in range(self.count)]
        for k, c in enumerate(got):
            if not ck.same_problem(c, self.params[k], A.YH_MODEL_FK3V,
                                   self.fks[k], self._masks[k]):
                check("yh_batch_load_checkpoint", A.YH_EINVAL)
        if len({c.step for c in got}) != 1 or not 0 <= got[0].step <= 2**31 - 1:
            check("yh_batch_load_checkpoint", A.YH_EINVAL)
        for k, c in enumerate(got):
            self.set_state(k, *c.fields)
        self.set_step(got[0].step)

    def launch_count(self):
        n = C.c_longlong()
        check("yh_batch_get_launch_count",
              self.lib.yh_batch_get_launch_count(self.h, C.byref(n)))
        return n.value
