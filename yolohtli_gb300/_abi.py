"""ctypes mirror of the structs and constants in include/yolohtli.h.

Pure type definitions: importing this module loads no library. The struct
layouts follow the C header, which mirrors the reference's typeDefinition.cuh
(paramVar :35-125, vec5dyn :19-20, stateVar :7-9).
"""
import ctypes as C

YH_OK = 0
YH_EINVAL = -1
YH_ECUDA = -2
YH_ENOMEM = -3
YH_ESINGULAR = -4
YH_ENONFINITE = -5
YH_EOVERFLOW = -6
YH_EUNSUPPORTED = -7
YH_ENOTREADY = -8
YH_ETIMEOUT = -9
YH_ECORRUPT = -10

STATUS_NAMES = {
    YH_OK: "YH_OK", YH_EINVAL: "YH_EINVAL", YH_ECUDA: "YH_ECUDA",
    YH_ENOMEM: "YH_ENOMEM", YH_ESINGULAR: "YH_ESINGULAR",
    YH_ENONFINITE: "YH_ENONFINITE", YH_EOVERFLOW: "YH_EOVERFLOW",
    YH_EUNSUPPORTED: "YH_EUNSUPPORTED", YH_ENOTREADY: "YH_ENOTREADY",
    YH_ETIMEOUT: "YH_ETIMEOUT", YH_ECORRUPT: "YH_ECORRUPT",
}

YH_ENGINE_STEP = 0
YH_ENGINE_BLOCKED = 1
YH_ENGINE_RESIDENT = 2
ENGINE_NAMES = {YH_ENGINE_STEP: "step", YH_ENGINE_BLOCKED: "blocked",
                YH_ENGINE_RESIDENT: "resident"}

YH_MODEL_REF2V = 0
YH_MODEL_FK3V = 1
YH_TEMPLATE_CURRENT = 0
YH_TEMPLATE_FROZEN = 1

NFIELDS = {YH_MODEL_REF2V: 2, YH_MODEL_FK3V: 3}


class Int2(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int)]


class Float2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


_B, _I, _D, _F = C.c_bool, C.c_int, C.c_double, C.c_float

# (name, ctype, alignment) in declaration order of paramVar.
_PARAM_FIELDS = (
    [(n, _B, 1) for n in (
        "animate", "saveEveryIt", "plotTip", "recordTip", "plotContour",
        "recordContour", "stimulate", "apdContour", "plotTimeSeries",
        "recordTimeSeries", "reduceSym", "reduceSymStart", "clock",
        "counterclock", "firstIterTip", "firstIterContour", "firstFPS",
        "solidSwitch", "neumannBC", "gateDiff", "anisotropy", "tipGrad")]
    + [(n, _I, 4) for n in ("lap4", "contourMode", "timeIntOrder", "tipAlgorithm")]
    + [(n, _B, 1) for n in ("load", "save")]
    + [(n, _I, 4) for n in ("nx", "ny", "memSize")]
    + [(n, _D, 8) for n in (
        "Lx", "Ly", "hx", "hy", "dt", "diff_par", "diff_per", "Dxx", "Dyy",
        "Dxy", "rx", "ry", "rxy", "rbx", "rby", "rscale", "invdx", "invdy",
        "sample")]
    + [("count", _I, 4), ("physicalTime", _D, 8), ("physicalTimeLim", _D, 8),
       ("startRecTime", _I, 4), ("stimPeriod", _D, 8), ("stimDuration", _D, 8),
       ("stimMag", _D, 8), ("fibThreshold", _B, 1), ("fibTerminated", _B, 1),
       ("leapShocks", _I, 4), ("eSize", _I, 4), ("point", Int2, 8),
       ("nc", _I, 4), ("rdomTrapz", _D, 8), ("rdomStim", _D, 8),
       ("rdomAPD", _D, 8), ("stcx", _D, 8), ("stcy", _D, 8),
       ("pointStim", Float2, 8), ("savePackage", _I, 4), ("tiempo", _F, 4),
       ("degrad", _D, 8), ("boundaryVal", _D, 8), ("qx4", _D, 8),
       ("qy4", _D, 8), ("fx4", _D, 8), ("fy4", _D, 8), ("itPerFrame", _I, 4),
       ("tipOffsetX", _I, 4), ("tipOffsetY", _I, 4), ("minVarColor", _F, 4),
       ("maxVarColor", _F, 4), ("wnx", _I, 4), ("wny", _I, 4),
       ("uMax", _F, 4), ("uMin", _F, 4), ("vMax", _F, 4), ("vMin", _F, 4),
       ("tipx", _F, 4), ("tipy", _F, 4)]
    + [(n, _D, 8) for n in (
        "contourThresh1", "contourThresh2", "contourThresh3", "Uth", "tc",
        "alpha", "beta", "gamma", "delta", "eps", "mu", "theta")]
)


def _laid_out(fields):
    """_fields_ with explicit padding under _pack_=1, applying the C rule
    (each member at a multiple of its alignment, size a multiple of the
    largest alignment) with CUDA's 8-byte int2/float2."""
    out, off, maxal, npad = [], 0, 1, 0
    for name, ct, al in fields:
        pad = (-off) % al
        if pad:
            out.append(("_pad%d" % npad, C.c_char * pad))
            npad += 1
            off += pad
        out.append((name, ct))
        off += C.sizeof(ct)
        maxal = max(maxal, al)
    pad = (-off) % maxal
    if pad:
        out.append(("_pad%d" % npad, C.c_char * pad))
    return out


class ParamVar(C.Structure):
    """yh_param_var == the reference's paramVar (typeDefinition.cuh:35-125)."""
    _pack_ = 1
    _fields_ = _laid_out(_PARAM_FIELDS)

    def copy(self):
        q = ParamVar()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(self))
        return q


PARAM_FIELD_NAMES = [f[0] for f in _PARAM_FIELDS]


class FKParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "tau_d", "tau_r", "tau_si", "tau_0", "tau_v_plus", "tau_v1_minus",
        "tau_v2_minus", "tau_w_plus", "tau_w_minus", "u_c", "u_v", "u_csi", "k")]


FK_NAMES = [f[0] for f in FKParams._fields_]


class Tip(C.Structure):
    """yh_tip == vec5dyn (typeDefinition.cuh:19-20)."""
    _fields_ = [(n, C.c_float) for n in ("x", "y", "vx", "vy", "t")]


class Fields(C.Structure):
    """yh_fields: device pointers u, v, w (stateVar plus w)."""
    _fields_ = [("u", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p)]


class Fields64(C.Structure):
    """yh_fields64: FP64 device pointers u, v, w."""
    _fields_ = [("u", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p)]


class SymState(C.Structure):
    _fields_ = [("c", C.c_double * 3), ("phi", C.c_double * 3),
                ("c_adv", C.c_double * 3), ("phi_adv", C.c_double * 3),
                ("integrals", C.c_double * 12), ("centre", C.c_float * 2),
                ("step", C.c_int), ("status", C.c_int), ("ntips", C.c_int),
                ("nsingular", C.c_int)]


class Stim(C.Structure):
    _fields_ = [("step", C.c_int), ("i0", C.c_int), ("j0", C.c_int),
                ("i1", C.c_int), ("j1", C.c_int), ("value", C.c_float)]


class ContourPt(C.Structure):
    """yh_contour_pt == the reference's float3 contour point."""
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("t", C.c_float)]


class ApdFields(C.Structure):
    """yh_apd_fields: device pointers of the space-APD tracker."""
    _fields_ = [(n, C.c_void_p) for n in ("apd1", "apd2", "sapd", "dapd",
                                           "back", "front", "first")]


class BatchStim(C.Structure):
    """yh_batch_stim: a stimulus event of one instance of a batch."""
    _fields_ = [("instance", C.c_int), ("s", Stim)]


class CheckpointHeader(C.Structure):
    """yh_checkpoint_header: the sizes a checkpoint file holds."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("model", C.c_int),
                ("nfields", C.c_int), ("has_mask", C.c_int),
                ("step", C.c_longlong)]


def param_defaults(nx, ny):
    """The reference's defaults (saveFiles.cu:105-231) for an nx x ny grid,
    with the derived coefficients of main.cu:148-158 (dt not halved).
    Host-side restatement; the library's yh_param_defaults computes the same."""
    import math
    p = ParamVar()
    p.animate = True
    p.plotTip = True
    p.plotTimeSeries = True
    p.neumannBC = True
    p.gateDiff = True
    p.tipAlgorithm = 1
    p.contourMode = 3
    p.lap4 = 0              # 5-point (the reference default is 4th order)
    p.timeIntOrder = 1      # Euler (the reference default is RK4)
    p.counterclock = True
    p.firstFPS = True
    p.firstIterTip = True
    p.firstIterContour = True
    p.nx, p.ny = nx, ny
    p.Lx = 12.0
    p.Ly = 12.0
    p.hx = p.Lx / (nx - 1.0)
    p.hy = p.Ly / (ny - 1.0)
    p.dt = 0.02
    p.diff_par = 0.001
    p.diff_per = 0.001
    th = p.degrad * 3.14159265359 / 180.0
    p.Dxx = p.diff_par * math.cos(th) ** 2 + p.diff_per * math.sin(th) ** 2
    p.Dyy = p.diff_par * math.sin(th) ** 2 + p.diff_per * math.cos(th) ** 2
    p.Dxy = (p.diff_par - p.diff_per) * math.sin(th) * math.cos(th)
    p.rscale = 0.01
    p.physicalTimeLim = 100000.0
    p.eSize = 2
    p.point.x, p.point.y = nx // 2, ny // 2
    p.stimPeriod = 600.0
    p.stimMag = 2.0
    p.stimDuration = 10.0
    p.fibThreshold = True
    p.nc = 100
    p.stcx = 0.25 * p.Lx
    p.stcy = 0.25 * p.Ly
    p.rdomStim = 0.03 * p.Lx
    p.rdomAPD = 0.15 * p.Lx
    p.tipOffsetX = 160
    p.tipOffsetY = 160
    p.rdomTrapz = 0.5 * ((p.tipOffsetX + p.tipOffsetY) * p.hx)
    p.itPerFrame = 50
    p.sample = 2.0
    p.minVarColor, p.maxVarColor = -0.1, 1.1
    p.wnx, p.wny = nx, ny
    p.uMin, p.uMax, p.vMin, p.vMax = -0.1, 1.1, -0.1, 0.5
    p.contourThresh1, p.contourThresh2, p.contourThresh3 = 0.8, 0.85, 0.7
    p.Uth = 0.7
    p.tc = 1.0
    p.alpha, p.beta, p.gamma, p.delta = 0.2, 1.1, 0.0, 1.0
    p.eps, p.mu, p.theta = 0.005, 1.0, 0.0
    param_derive(p)
    return p


def param_derive(p):
    """Derived coefficients (main.cu:149-155, saveFiles.cu:157-170)."""
    p.rx = p.dt * p.Dxx / (p.hx * p.hx)
    p.ry = p.dt * p.Dyy / (p.hy * p.hy)
    p.rxy = 2.0 * p.Dxy * p.dt / (4.0 * p.hx * p.hy)
    p.rbx = p.hx * p.Dxy / (p.Dxx * p.hy) if p.Dxx else 0.0
    p.rby = p.hy * p.Dxy / (p.Dyy * p.hx) if p.Dyy else 0.0
    p.invdx = 0.5 / p.hx
    p.invdy = 0.5 / p.hy
    p.qx4 = p.dt * p.Dyy / (p.hy * p.hy * 12.0)
    p.qy4 = p.dt * p.Dxx / (p.hx * p.hx * 12.0)
    p.fx4 = p.dt / 12.0
    p.fy4 = p.dt / 12.0
    p.memSize = p.nx * p.ny * 8
    return p


def fk_defaults():
    """Fenton-Karma 1998 'BR' fit (the parameter set of the FK3V workloads)."""
    fk = FKParams()
    fk.tau_d, fk.tau_r, fk.tau_si, fk.tau_0 = 0.25, 50.0, 45.0, 8.3
    fk.tau_v_plus, fk.tau_v1_minus, fk.tau_v2_minus = 3.33, 19.6, 1000.0
    fk.tau_w_plus, fk.tau_w_minus = 667.0, 11.0
    fk.u_c, fk.u_v, fk.u_csi, fk.k = 0.13, 0.055, 0.85, 10.0
    return fk


def fk_tissue_params(nx, ny, dx=0.025, D=0.001, dt=0.05):
    """Parameters of the FK3V tissue workloads: square cells of side dx (cm),
    isotropic D (cm^2/ms), time step dt (ms); D*dt/dx^2 = 0.08 by default."""
    p = param_defaults(nx, ny)
    p.hx = p.hy = dx
    p.Lx = dx * (nx - 1)
    p.Ly = dx * (ny - 1)
    p.dt = dt
    p.diff_par = p.diff_per = D
    p.Dxx = p.Dyy = D
    p.Dxy = 0.0
    p.gateDiff = False
    return param_derive(p)
