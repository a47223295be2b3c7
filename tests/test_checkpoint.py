"""This library's binary checkpoint file, on the CPU: round trips, the byte
layout the header declares (restated here in Python), and corrupted or
truncated files, which the reader reports as YH_ECORRUPT. Faults are
injected on the host, into the file."""
import ctypes as C
import struct

import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import checkpoint as ck
from yolohtli_gb300 import load
from yolohtli_gb300.ops import YolohtliError


def fnv1a64(data):
    h = 0xcbf29ce484222325
    for b in data:
        h = ((h ^ b) * 0x100000001b3) & 0xffffffffffffffff
    return h


def _case(model, nx=23, ny=17, mask=True, seed=0):
    rng = np.random.default_rng(seed)
    p = A.fk_tissue_params(nx, ny)
    n = nx * ny
    nf = A.NFIELDS[model]
    fields = [rng.standard_normal(n).astype(np.float32) for _ in range(nf)]
    m = (rng.random(n) > 0.2).astype(np.uint8) if mask else None
    return p, A.fk_defaults(), fields, m


@pytest.mark.parametrize("model,mask", [(A.YH_MODEL_FK3V, True),
                                        (A.YH_MODEL_FK3V, False),
                                        (A.YH_MODEL_REF2V, True),
                                        (A.YH_MODEL_REF2V, False)])
def test_round_trip_is_exact(tmp_path, model, mask):
    p, fk, fields, m = _case(model, mask=mask)
    path = tmp_path / "state.yhck"
    ck.write(path, p, model, fk, 12345, *fields, mask=m)
    h = ck.header(path)
    assert (h.nx, h.ny, h.model, h.nfields, h.has_mask, h.step) == (
        p.nx, p.ny, model, len(fields), int(mask), 12345)
    r = ck.read(path)
    assert r.model == model and r.step == 12345
    assert bytes(r.p) == bytes(p)
    if model == A.YH_MODEL_FK3V:
        assert bytes(r.fk) == bytes(fk)
    for a, b in zip(r.fields, fields):
        assert a.tobytes() == b.tobytes()
    if mask:
        assert np.array_equal(r.mask, m)
    else:
        assert r.mask is None


def test_byte_layout_and_hash(tmp_path):
    """The header fields at the offsets include/yolohtli.h gives, and the
    FNV-1a 64-bit hash of the payload, computed here independently."""
    p, fk, fields, m = _case(A.YH_MODEL_FK3V, nx=9, ny=7)
    path = tmp_path / "s.yhck"
    ck.write(path, p, A.YH_MODEL_FK3V, fk, 77, *fields, mask=m)
    raw = path.read_bytes()
    head, payload = raw[:64], raw[64:]
    assert head[:8] == b"YHCKPT\0\0"
    version, bom, nx, ny, model, nf, has_mask, pbytes, step, size, hsh = \
        struct.unpack_from("<IIiiiiiiqQQ", head, 8)
    assert (version, bom) == (1, 0x01020304)
    assert (nx, ny, model, nf, has_mask, step) == (9, 7, 1, 3, 1, 77)
    assert pbytes == C.sizeof(A.ParamVar)
    expect = (bytes(p) + bytes(fk) + m.tobytes() +
              b"".join(f.tobytes() for f in fields))
    assert size == len(payload) and payload == expect
    assert hsh == fnv1a64(payload)


def _status(fn):
    with pytest.raises(YolohtliError) as e:
        fn()
    return e.value.status


def _mutate(path, out, edit):
    raw = bytearray(path.read_bytes())
    raw = edit(raw)
    out.write_bytes(bytes(raw))
    return out


def _flip(offset):
    def edit(raw):
        raw[offset] ^= 0x10
        return raw
    return edit


@pytest.mark.parametrize("name,edit", [
    ("magic", _flip(0)),
    ("version", _flip(8)),
    ("byte order", _flip(13)),
    ("model", lambda r: r[:24] + struct.pack("<i", 5) + r[28:]),
    ("nfields", lambda r: r[:28] + struct.pack("<i", 2) + r[32:]),
    ("mask flag", lambda r: r[:32] + struct.pack("<i", 0) + r[36:]),
    ("step", lambda r: r[:40] + struct.pack("<q", -1) + r[48:]),
    ("payload size", _flip(48)),
    ("hash", _flip(60)),
    ("a parameter byte", _flip(64 + 100)),
    ("a mask byte", _flip(64 + C.sizeof(A.ParamVar) + 104 + 5)),
    ("the last field byte", lambda r: r[:-1] + bytes([r[-1] ^ 1])),
    ("truncated header", lambda r: r[:40]),
    ("truncated payload", lambda r: r[:-3]),
    ("a trailing byte", lambda r: r + b"\0"),
])
def test_corruption_is_reported(tmp_path, name, edit):
    p, fk, fields, m = _case(A.YH_MODEL_FK3V)
    good = tmp_path / "good.yhck"
    ck.write(good, p, A.YH_MODEL_FK3V, fk, 5, *fields, mask=m)
    bad = _mutate(good, tmp_path / "bad.yhck", edit)
    assert _status(lambda: ck.read(bad)) == A.YH_ECORRUPT, name


def test_header_checks_need_no_payload_read(tmp_path):
    """The header reader checks the header alone: a payload flip passes it
    and fails the full read."""
    p, fk, fields, m = _case(A.YH_MODEL_REF2V)
    good = tmp_path / "good.yhck"
    ck.write(good, p, A.YH_MODEL_REF2V, None, 0, *fields, mask=m)
    bad = _mutate(good, tmp_path / "bad.yhck", _flip(200))
    assert ck.header(bad).step == 0
    assert _status(lambda: ck.read(bad)) == A.YH_ECORRUPT


def test_bad_arguments(tmp_path):
    lib = load()
    p, fk, fields, m = _case(A.YH_MODEL_FK3V)
    u, v, w = fields
    path = str(tmp_path / "x.yhck").encode()
    # FK3V needs its parameters and w; the step is not negative
    assert lib.yh_write_checkpoint(path, C.byref(p), A.YH_MODEL_FK3V, None, None,
                                   0, u.ctypes.data, v.ctypes.data,
                                   w.ctypes.data) == A.YH_EINVAL
    assert lib.yh_write_checkpoint(path, C.byref(p), A.YH_MODEL_FK3V,
                                   C.byref(fk), None, 0, u.ctypes.data,
                                   v.ctypes.data, None) == A.YH_EINVAL
    assert lib.yh_write_checkpoint(path, C.byref(p), A.YH_MODEL_FK3V,
                                   C.byref(fk), None, -1, u.ctypes.data,
                                   v.ctypes.data, w.ctypes.data) == A.YH_EINVAL
    assert lib.yh_write_checkpoint(path, C.byref(p), 9, C.byref(fk), None, 0,
                                   u.ctypes.data, v.ctypes.data,
                                   w.ctypes.data) == A.YH_EINVAL
    # a missing file and a directory are argument errors, not corruption
    missing = str(tmp_path / "none.yhck").encode()
    h = A.CheckpointHeader()
    assert lib.yh_read_checkpoint_header(missing, C.byref(h)) == A.YH_EINVAL
    assert lib.yh_write_checkpoint(str(tmp_path).encode(), C.byref(p),
                                   A.YH_MODEL_FK3V, C.byref(fk), None, 0,
                                   u.ctypes.data, v.ctypes.data,
                                   w.ctypes.data) == A.YH_EINVAL
    assert lib.yh_read_checkpoint(None, None, None, None, None, None, None,
                                  None, None) == A.YH_EINVAL


def test_status_strings_of_the_failure_codes():
    lib = load()
    assert lib.yh_status_string(A.YH_ETIMEOUT) == b"device-side wait timed out"
    assert lib.yh_status_string(A.YH_ECORRUPT) == b"corrupt checkpoint file"
    assert lib.yh_status_string(A.YH_ENONFINITE) == b"non-finite state"


def test_same_problem_is_the_load_rule(tmp_path):
    p, fk, fields, m = _case(A.YH_MODEL_FK3V)
    path = tmp_path / "s.yhck"
    ck.write(path, p, A.YH_MODEL_FK3V, fk, 3, *fields, mask=m)
    c = ck.read(path)
    assert ck.same_problem(c, p, A.YH_MODEL_FK3V, fk, m)
    assert ck.same_problem(c, p, A.YH_MODEL_FK3V, fk, m * 7)  # nonzero = tissue
    q = p.copy()
    q.Lx += 1.0   # not a step coefficient
    assert ck.same_problem(c, q, A.YH_MODEL_FK3V, fk, m)
    q = p.copy()
    q.rx *= 1.5
    assert not ck.same_problem(c, q, A.YH_MODEL_FK3V, fk, m)
    f2 = A.fk_defaults()
    f2.k = 11.0
    assert not ck.same_problem(c, p, A.YH_MODEL_FK3V, f2, m)
    m2 = m.copy()
    m2[0] = 1 - m2[0]
    assert not ck.same_problem(c, p, A.YH_MODEL_FK3V, fk, m2)
    assert not ck.same_problem(c, p, A.YH_MODEL_FK3V, fk, None)
    assert not ck.same_problem(c, p, A.YH_MODEL_REF2V, fk, m)


@pytest.mark.parametrize("field", ["nx", "ny", "gateDiff", "rx", "ry", "rscale",
                                   "dt", "tc", "mu", "alpha", "eps", "delta",
                                   "gamma", "beta", "theta"])
def test_same_problem_covers_every_step_coefficient(field):
    """Every input of the step coefficients decides whether a checkpoint
    belongs to a handle (yh_checkpoint_same_problem, the C rule the single
    grid and the batch both use)."""
    lib = load()
    p, fk, _, _ = _case(A.YH_MODEL_FK3V)
    q = p.copy()
    v = getattr(q, field)
    setattr(q, field, (not v) if isinstance(v, bool) else v + 1)
    same = lambda a, b: lib.yh_checkpoint_same_problem(
        C.byref(a), A.YH_MODEL_FK3V, C.byref(fk), C.byref(b),
        A.YH_MODEL_FK3V, C.byref(fk))
    assert same(p, p) == 1
    assert same(p, q) == 0


def test_write_replaces_the_file_only_when_complete(tmp_path):
    """A save goes to path.tmp and is renamed over path: a failed write
    leaves the earlier file in place and no temporary behind."""
    p, fk, fields, m = _case(A.YH_MODEL_FK3V)
    path = tmp_path / "s.yhck"
    ck.write(path, p, A.YH_MODEL_FK3V, fk, 3, *fields, mask=m)
    good = path.read_bytes()
    # a directory in place of the temporary file makes the write fail
    (tmp_path / "s.yhck.tmp").mkdir()
    with pytest.raises(YolohtliError):
        ck.write(path, p, A.YH_MODEL_FK3V, fk, 4, *fields, mask=m)
    assert path.read_bytes() == good
    (tmp_path / "s.yhck.tmp").rmdir()
    ck.write(path, p, A.YH_MODEL_FK3V, fk, 4, *fields, mask=m)
    assert ck.read(path).step == 4
    assert sorted(x.name for x in tmp_path.iterdir()) == ["s.yhck"]
