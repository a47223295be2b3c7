"""Python host layer over the C ABI (include/yolohtli.h).

Stateless operators take torch CUDA tensors (FP32, flat, nx*ny) and call the
library on torch's current stream; the solver handle is in solver.py. Every
call raises YolohtliError on a non-zero status: there is no fallback path.
"""
import ctypes as C

from . import _abi as A
from ._loader import load


class YolohtliError(RuntimeError):
    def __init__(self, fn, status):
        self.status = status
        super().__init__("%s failed: %s (%d)" % (
            fn, A.STATUS_NAMES.get(status, "?"), status))


def check(fn, status):
    if status != A.YH_OK:
        raise YolohtliError(fn, status)
    return status


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return None if t is None else t.data_ptr()


def fields(ts):
    """yh_fields from a list of 2 or 3 tensors (or None)."""
    f = A.Fields()
    if ts is None:
        return f
    f.u = _p(ts[0])
    f.v = _p(ts[1])
    f.w = _p(ts[2]) if len(ts) > 2 else None
    return f


def reaction_diffusion(p, model, fk, out, inp, vel_tan=None, solid=None):
    """One Euler step out <- inp (lists of FP32 tensors); replaces
    reactionDiffusion_wrapper (hostPrototypes.h:22-25)."""
    lib = load()
    return check("yh_reaction_diffusion", lib.yh_reaction_diffusion(
        C.byref(p), model, C.byref(fk) if fk is not None else None,
        fields(out), fields(inp), fields(vel_tan), _p(solid), _stream()))


def spiral_tip(p, past_u, present_u, tip_count, tip_vec, capacity,
               physical_time=0.0, solid=None):
    """Tip detection; tip_count (int32[1]) and tip_vec (float32[5*cap])."""
    lib = load()
    return check("yh_spiral_tip", lib.yh_spiral_tip(
        C.byref(p), _p(past_u), _p(present_u), C.c_double(physical_time),
        _p(tip_count), _p(tip_vec), capacity, _p(solid), _stream()))


def filament_mark(p, past_u, present_u, mark):
    """tipAlgorithm 3: sets mark (uint8, nx*ny) on the filament cells."""
    return check("yh_filament_mark", load().yh_filament_mark(
        C.byref(p), _p(past_u), _p(present_u), _p(mark), _stream()))


def contour(p, field1, field2, stim_area, mode, time, count, vec, capacity,
            plot=None):
    """Contour points (modes 1-3) into vec (float32[3*capacity])."""
    return check("yh_contour", load().yh_contour(
        C.byref(p), _p(field1), _p(field2), _p(stim_area), int(mode),
        C.c_float(time), _p(count), _p(vec), int(capacity), _p(plot),
        _stream()))


def space_apd(p, count, uold, unew, apd, stim_area=None, stimulate=False):
    """One step of the space-APD tracker; apd: dict of device tensors
    apd1, apd2, sapd, dapd, back, front (float32) and first (uint8)."""
    f = A.ApdFields(*[_p(apd[k]) if apd.get(k) is not None else None
                      for k in ("apd1", "apd2", "sapd", "dapd", "back",
                                "front", "first")])
    return check("yh_space_apd", load().yh_space_apd(
        C.byref(p), int(count), _p(uold), _p(unew), f, _p(stim_area),
        1 if stimulate else 0, _stream()))


def pick_centre(tip_count, tip_vec, capacity, sym):
    lib = load()
    return check("yh_pick_centre", lib.yh_pick_centre(
        _p(tip_count), _p(tip_vec), capacity, _p(sym), _stream()))


def phase_workspace_bytes(nx, ny):
    return load().yh_phase_integrals_workspace(nx, ny)


def phase_integrals(p, model, state, vel_tan, adv_rows, adv_cols, sym,
                    workspace, templ=None, solid=None):
    """Fused slices + 12 FP64 integrals + FP64 solve into `sym` (a device
    yh_sym_state, e.g. a uint8 tensor of sizeof bytes)."""
    lib = load()
    tx = fields(templ[0]) if templ else A.Fields()
    ty = fields(templ[1]) if templ else A.Fields()
    tt = fields(templ[2]) if templ else A.Fields()
    return check("yh_phase_integrals", lib.yh_phase_integrals(
        C.byref(p), model, fields(state), fields(vel_tan), tx, ty, tt,
        _p(adv_rows), _p(adv_cols), _p(solid), _p(sym), _p(workspace),
        _stream()))


def template_slices(p, model, state, tx, ty, tt):
    lib = load()
    return check("yh_template_slices", lib.yh_template_slices(
        C.byref(p), model, fields(state), fields(tx), fields(ty), fields(tt),
        _stream()))


def comoving_field(p, sym, adv_rows, adv_cols, adv_rows_f=None,
                   adv_cols_f=None, advance=False):
    lib = load()
    return check("yh_comoving_field", lib.yh_comoving_field(
        C.byref(p), _p(sym), _p(adv_rows), _p(adv_cols), _p(adv_rows_f),
        _p(adv_cols_f), 1 if advance else 0, _stream()))


def advect_bfecc(p, model, out, inp, adv_rows_f, adv_cols_f, uf, ue,
                 solid=None, three_launches=False):
    lib = load()
    name = "yh_advect_bfecc_3pass" if three_launches else "yh_advect_bfecc"
    return check(name, getattr(lib, name)(
        C.byref(p), model, fields(out), fields(inp), _p(adv_rows_f),
        _p(adv_cols_f), _p(solid), fields(uf), fields(ue), _stream()))


def sym_advance(p, sym):
    return check("yh_sym_advance", load().yh_sym_advance(
        C.byref(p), _p(sym), _stream()))


def stimulate_box(p, u, i0, j0, i1, j1, value, solid=None):
    return check("yh_stimulate_box", load().yh_stimulate_box(
        C.byref(p), _p(u), _p(solid), i0, j0, i1, j1, C.c_float(value),
        _stream()))


def sym_from_bytes(t):
    """A host SymState from a device uint8 tensor holding a yh_sym_state."""
    raw = bytes(t.cpu().numpy().tobytes())
    s = A.SymState()
    C.memmove(C.byref(s), raw, C.sizeof(s))
    return s


def sym_to_tensor(s, device="cuda"):
    import torch
    buf = (C.c_uint8 * C.sizeof(s)).from_buffer_copy(s)
    return torch.tensor(list(buf), dtype=torch.uint8, device=device)


def fields64(ts):
    """yh_fields64 from a list of 2 or 3 FP64 tensors (or None)."""
    f = A.Fields64()
    if ts is None:
        return f
    f.u = _p(ts[0])
    f.v = _p(ts[1])
    f.w = _p(ts[2]) if len(ts) > 2 else None
    return f


def reaction_diffusion_f64(p, model, fk, out, inp, vel_tan=None, solid=None):
    """reaction_diffusion on FP64 tensors: the same kernel in double."""
    return check("yh_reaction_diffusion_f64", load().yh_reaction_diffusion_f64(
        C.byref(p), model, C.byref(fk) if fk is not None else None,
        fields64(out), fields64(inp), fields64(vel_tan), _p(solid),
        _stream()))


def spiral_tip_f64(p, past_u, present_u, tip_count, tip_vec, capacity,
                   physical_time=0.0, solid=None):
    """spiral_tip on FP64 u levels (tips are FP32 yh_tip records)."""
    return check("yh_spiral_tip_f64", load().yh_spiral_tip_f64(
        C.byref(p), _p(past_u), _p(present_u), C.c_double(physical_time),
        _p(tip_count), _p(tip_vec), capacity, _p(solid), _stream()))


def stimulate_box_f64(p, u, i0, j0, i1, j1, value, solid=None):
    return check("yh_stimulate_box_f64", load().yh_stimulate_box_f64(
        C.byref(p), _p(u), _p(solid), i0, j0, i1, j1, C.c_double(value),
        _stream()))
