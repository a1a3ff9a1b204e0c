"""The step kernel's cheap reject (`near_pair`, device.cuh) never drops a
pair the reference keeps.

The reference's contact test is `sqrt(d.d) < ra + rb` in f32
(physics.rs:264-269).  Before it, the kernels reject a candidate when
`D > T` with `D = dx*dx + dy*dy` and `T = (m*m) * 1.00000024f`, m = ra + rb,
every operation rounded to f32 (compiled with --fmad=false).  T is at least
m^2 in real arithmetic (the factor 1 + 2^-22 outweighs the two roundings),
so D > T implies sqrt(D) > m, and the rounded square root is then at least
m: the reference rejects as well.  This file restates the arithmetic in
NumPy float32 and checks the implication on random and on adversarial
pairs placed within a few ulps of the contact boundary.
"""
import os

import numpy as np

F = np.float32


def near_pair(dx, dy, m):
    """device.cuh near_pair, in f32 (no fused operations)."""
    d = (dx * dx) + (dy * dy)
    t = (m * m) * F(1.00000024)
    return ~(d > t)


def reference_contact(dx, dy, m):
    """physics.rs:264-269: sqrt(axis.dot(axis)) < min_dist, in f32."""
    return np.sqrt((dx * dx) + (dy * dy)) < m


def test_margin_constant_is_one_plus_two_to_the_minus_22():
    assert F(1.00000024) == F(1.0) + F(2.0 ** -22)
    # the restatement above is the kernels' own arithmetic
    src = open(os.path.join(os.path.dirname(__file__), "..", "blobs_gb300", "csrc", "device.cuh")).read()
    assert "const float D = (dx * dx) + (dy * dy);" in src
    assert "const float T = (mind * mind) * 1.00000024f;" in src


def _check(dx, dy, m):
    dx, dy, m = dx.astype(np.float32), dy.astype(np.float32), m.astype(np.float32)
    keep = near_pair(dx, dy, m)
    ref = reference_contact(dx, dy, m)
    missed = ref & ~keep
    assert not missed.any(), (dx[missed][:3], dy[missed][:3], m[missed][:3])
    return keep, ref


def test_never_rejects_a_reference_contact_random():
    rng = np.random.Generator(np.random.PCG64(11))
    n = 2_000_000
    m = rng.uniform(1e-3, 10.0, n)
    r = m * rng.uniform(0.0, 2.0, n)
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    keep, ref = _check(r * np.cos(th), r * np.sin(th), m)
    assert ref.sum() > n // 3 and (keep & ~ref).sum() < n // 1000  # the pre-test is tight


def test_never_rejects_a_reference_contact_at_the_boundary():
    """Distances within +-64 ulps of m, at many scales and angles, including
    axis-aligned pairs (dy = 0) where d.d is a single rounded square."""
    rng = np.random.Generator(np.random.PCG64(12))
    n = 400_000
    m = F(np.exp(rng.uniform(np.log(1e-4), np.log(1e4), n)))
    k = rng.integers(-64, 65, n)
    r = m.astype(np.float64) * (1.0 + k.astype(np.float64) * 2.0 ** -24)  # about k ulps from m
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    th[: n // 4] = 0.0
    keep, ref = _check(r * np.cos(th), r * np.sin(th), m)
    assert ref.any() and (~ref).any()
    # every exact-boundary candidate the reference accepts is kept, and the
    # ones it drops are mostly dropped by the pre-test as well
    assert (keep & ~ref).mean() < 0.5


def test_exhaustive_axis_aligned_neighbourhood():
    """For m on a grid of f32 values, every dx within 256 ulps of m (dy = 0)."""
    ms = F(np.linspace(0.01, 5.0, 997))
    offs = np.arange(-256, 257)
    m = np.repeat(ms, len(offs))
    bits = m.view(np.int32) + np.tile(offs, len(ms)).astype(np.int32)
    dx = bits.view(np.float32)
    _check(dx, np.zeros_like(dx), m)
