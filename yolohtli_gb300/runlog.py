"""A JSON-lines run log for long solver runs: one line per segment.

The reference's only observability is a frames-per-second readout in the
GLUT window title (main.cu:1817-1847) and printf to stdout. Here, each line
of a plain run holds:
- the step reached and the segment's steps and wall seconds;
- Gcell-steps/s, and GB/s at the algorithmic bytes of a step (24 B per
  cell-step for FK3V, 16 for REF2V, plus 1 with a hole mask);
- the fraction of an HBM peak, when one is given;
- the tip count between the last two time levels;
- the number of non-finite state values.
A symmetry-reduced run logs c, phi, the solve status and the tip count
instead of tips and the finite check.

Errors against the oracle are not logged: the oracle is test
infrastructure, and the library does not ship it."""
import json
import time

from . import _abi as A

_BYTES_PER_CELL_STEP = {A.YH_MODEL_FK3V: 24, A.YH_MODEL_REF2V: 16}


def bytes_per_cell_step(model, has_mask):
    """Algorithmic bytes of one step per cell: read and write every field
    once, plus the 1-byte mask."""
    return _BYTES_PER_CELL_STEP[model] + (1 if has_mask else 0)


class RunLog:
    """Writes one JSON object per line to `out`: a path (opened for
    append) or a file object."""

    def __init__(self, out):
        self._own = isinstance(out, (str, bytes)) or hasattr(out, "__fspath__")
        self.f = open(out, "a") if self._own else out
        self.records = []

    def record(self, **fields):
        self.f.write(json.dumps(fields, sort_keys=True) + "\n")
        self.f.flush()
        self.records.append(fields)
        return fields

    def close(self):
        if self._own and self.f:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _timed(sim, fn):
    sim.synchronize()
    t0 = time.perf_counter()
    fn()
    sim.synchronize()
    return time.perf_counter() - t0


def run_logged(sim, nsteps, log, stims=(), every=1000, peak_gbs=None,
               tips=True, finite=True):
    """sim.run(nsteps, stims) in segments of `every` steps (a
    solver.Monodomain), one log line per segment; returns the lines.
    Tip tracking and the finite check run after the timed segment."""
    every = max(1, int(every))
    ncell = sim.p.nx * sim.p.ny
    bps = bytes_per_cell_step(sim.model, sim.has_mask)
    left, lines = int(nsteps), []
    while left > 0:
        m = min(every, left)
        sec = _timed(sim, lambda: sim.run(m, stims))
        rate = ncell * m / sec if sec > 0 else float("inf")
        rec = dict(mode="plain", step=sim.step_count(), steps=m,
                   seconds=round(sec, 6),
                   gcell_steps_per_s=round(rate / 1e9, 3),
                   gbps=round(rate * bps / 1e9, 1))
        if peak_gbs:
            rec["hbm_frac"] = round(rate * bps / 1e9 / peak_gbs, 3)
        if tips:
            sim.track_tips()
            rec["ntips"] = int(len(sim.get_tips()))
        if finite:
            rec["nonfinite"] = int(sim.check_finite())
        lines.append(log.record(**rec))
        left -= m
    return lines


def sr_logged(sim, nsteps, log, every=100):
    """sim.sr_step(nsteps) after sim.sr_begin(...), in segments of `every`
    steps, one log line per segment with the frame's c and phi."""
    every = max(1, int(every))
    left, lines = int(nsteps), []
    while left > 0:
        m = min(every, left)
        sec = _timed(sim, lambda: sim.sr_step(m))
        sym = sim.get_sym()
        lines.append(log.record(
            mode="sr", step=sim.step_count(), steps=m, seconds=round(sec, 6),
            sr_steps_per_s=round(m / sec, 1) if sec > 0 else None,
            c=[float(x) for x in sym.c], phi=[float(x) for x in sym.phi],
            status=A.STATUS_NAMES.get(sym.status, sym.status),
            ntips=int(sym.ntips)))
        left -= m
    return lines
