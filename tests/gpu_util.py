"""Helpers of the GPU tests: torch device buffers for the C ABI calls."""
import numpy as np


def dev(x, dtype=None):
    import torch
    dtype = dtype or torch.float32
    return torch.tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def host(t):
    return t.detach().cpu().numpy()


def zeros_like_fields(fs):
    import torch
    return [torch.zeros_like(f) for f in fs]


def rel_l2(a, b, mask=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def max_abs(a, b):
    return float(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).max())


def smooth_state(nx, ny, seed, nf=2):
    rng = np.random.default_rng(seed)
    jj, ii = np.mgrid[0:ny, 0:nx]
    out = []
    for f in range(nf):
        z = np.zeros((ny, nx))
        for _ in range(4):
            a, b = rng.uniform(0.05, 0.3, 2)
            z += 0.25 * np.sin(a * ii + b * jj + rng.uniform(0, 6))
        out.append((0.5 + z).ravel())
    return out


def tips_match(a, b, tol):
    """True if the tip sets (n x >=2 arrays of x, y) match within tol."""
    if len(a) != len(b):
        return False
    if len(a) == 0:
        return True
    a = a[np.lexsort((a[:, 0], a[:, 1]))]
    b = b[np.lexsort((b[:, 0], b[:, 1]))]
    return bool(np.abs(a[:, :2] - b[:, :2]).max() <= tol)
