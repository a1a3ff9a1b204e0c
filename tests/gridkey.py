"""NumPy restatement of the broadphase cell coordinate (blobs::grid_coord in
blobs_gb300/csrc/device.cuh), operation for operation in float32, so CPU
tests can enumerate the same cells the device does.

Below GRID_FAST_CELLS cells from the origin: floor(fl(fl(v - o) * inv)).
At or beyond it: floor((v - o) * inv) carried exactly -- v - o as s + e
(TwoSum), s * inv as p + r1 (the FMA residual, exact in float32 and
computed here in float64, where the product of two floats is exact).
"""
import numpy as np

GRID_FAST_CELLS = np.float32(32768.0)
I32_MAX, I32_MIN = 2147483647, -2147483648


def _floor_sat(q):
    f = np.floor(np.asarray(q, np.float64))
    out = np.where(np.isnan(f), 0.0, np.clip(f, I32_MIN, I32_MAX))
    return out.astype(np.int64)


def grid_coord(v, o, inv):
    f32 = np.float32
    with np.errstate(over="ignore", invalid="ignore"):
        v = np.asarray(v, f32)
        o, inv = f32(o), f32(inv)
        q = (v - o) * inv
        aq = np.abs(q)
        fast = (aq < GRID_FAST_CELLS) | ~(aq <= f32(3.402823466e38))
        out = _floor_sat(q)
        if np.any(~fast):
            vf = v[~fast] if v.ndim else v
            s = vf - o
            bb = s - vf
            e = (vf - (s - bb)) + ((-o) - bb)
            p = s * inv
            r1 = (s.astype(np.float64) * np.float64(inv) - p.astype(np.float64)).astype(f32)
            t = r1 + e * inv
            fl = np.floor(p)
            fg = np.clip(np.floor((p - fl) + t), f32(-1024.0), f32(1024.0))
            flc = np.clip(fl, f32(-4.0e18), f32(4.0e18))
            k = np.clip(flc.astype(np.float64).astype(np.int64) + fg.astype(np.int64), I32_MIN, I32_MAX)
            if v.ndim:
                out[~fast] = k
            else:
                out = k
    return out


def grid_coord_plain(v, o, inv):
    """The plain float32 formula alone (exact only near the origin)."""
    with np.errstate(over="ignore", invalid="ignore"):
        return _floor_sat((np.asarray(v, np.float32) - np.float32(o)) * np.float32(inv))
