"""Known-answer tests of the contact pass's pair order, computed by hand in f32.

The reference resolves contacts pair by pair, i (outer, higher collider
index) ascending and j < i ascending (physics.rs:244-249), each pair moving
both bodies by the mass-ratio correction (physics.rs:291-300):

    axis = s_a - s_b; d = |axis|; n = axis / d; delta = (r_a + r_b) - d
    ratio = 1 - m_a / (m_a + m_b)
    p_a += (ratio * delta) * n;  p_b -= ((1 - ratio) * delta) * n

so a body in several contacts receives its increments in ascending partner
index, and f32 addition does not commute.  Each scene below is one substep
(substeps = 1, dt = 1/60, zero velocity, no gravity) worked through pair by
pair in NumPy float32 -- written out here, not through the oracle's loop --
then update_objects (physics.rs:323-367: disp = (p - p_old) * (dt / old_dt)
with old_dt = 1 for the first dynamic body of a fresh world and dt after it;
p_old = p; p += disp + a dt dt; v = disp / dt).  The resulting bit patterns
are also kept as literals.

1. Three contacts on one body whose corrections round differently in any
   other order: the oracle and the GPU reproduce the reference order's bits.
2. A push-out pair (coincident centres, physics.rs:272-286) one of whose
   bodies already had a correction earlier in the same substep: the
   reference refreshes both snapshots from the corrected positions before it
   takes the axis; the GPU takes the axis from the positions at the start
   of the contact pass.  The oracle reproduces the reference's bits, the
   GPU the bits of its documented rule, and the two differ by the stated
   amount (PUSHOUT_DEVIATION).
"""
import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

F = np.float32
DT = 1.0 / 60.0

# scene 1: body 3 touches bodies 0, 1, 2 (which do not touch each other)
POS3 = np.array([[1.5000814199447632, 0.3467235565185547], [0.2269573211669922, 1.0438557863235474],
                 [0.2780238389968872, -0.6365472674369812], [0.8263578414916992, 0.2829224467277527]], F)
RAD3 = np.array([0.34287023544311523, 0.4516792595386505, 0.5864827632904053, 0.7087827920913696], F)

# scene 2: body 1 touches body 0; body 2 sits exactly on body 1 (push-out)
POS2 = np.array([[0.0, 0.0], [0.8, 0.05], [0.8, 0.05]], F)
RAD2 = np.array([0.5, 0.5, 0.1], F)


def mass(r):
    # the lone sphere's mass, (0 + 2r) + 2r (rigid_body.rs:96-128, doubled handle)
    return F(F(F(0.0) + F(F(2.0) * r)) + F(F(2.0) * r))


def v2(x, y):
    return np.array([x, y], F)


def correction(sa, sb, ra, rb, ma, mb):
    """The pair's increments of p_a and p_b (physics.rs:264-300, no push-out)."""
    ax = v2(sa[0] - sb[0], sa[1] - sb[1])
    d = F(np.sqrt(F(F(ax[0] * ax[0]) + F(ax[1] * ax[1]))))
    n = v2(ax[0] / d, ax[1] / d)
    delta = F(F(ra + rb) - d)
    ratio = F(F(1.0) - F(ma / F(ma + mb)))
    ka, kb = F(ratio * delta), F(F(F(1.0) - ratio) * delta)
    return v2(F(ka * n[0]), F(ka * n[1])), v2(F(kb * n[0]), F(kb * n[1]))


def update_objects(p, p_start):
    """physics.rs:323-367 for zero velocity, no force, fresh world (old_dt 1)."""
    dt = F(F(DT) / F(1.0))
    pos, pold, vel = [], [], []
    old_dt = F(1.0)
    for b in range(len(p)):
        ratio = F(dt / old_dt)
        old_dt = dt
        disp = v2(F(F(p[b][0] - p_start[b][0]) * ratio), F(F(p[b][1] - p_start[b][1]) * ratio))
        acc = v2(F(F(F(0.0) * dt) * dt), F(F(F(0.0) * dt) * dt))
        pos.append(v2(F(p[b][0] + F(disp[0] + acc[0])), F(p[b][1] + F(disp[1] + acc[1]))))
        pold.append(p[b].copy())
        vel.append(v2(F(disp[0] / dt), F(disp[1] / dt)))
    return np.array(pos), np.array(pold), np.array(vel)


def hand_three(order=(0, 1, 2)):
    m = [mass(r) for r in RAD3]
    p = [x.copy() for x in POS3]
    s = POS3  # snapshots at the start of the contact pass
    for j in order:  # the reference visits (3, 0), (3, 1), (3, 2)
        ca, cb = correction(s[3], s[j], RAD3[3], RAD3[j], m[3], m[j])
        p[3] = v2(F(p[3][0] + ca[0]), F(p[3][1] + ca[1]))
        p[j] = v2(F(p[j][0] - cb[0]), F(p[j][1] - cb[1]))
    return update_objects(p, POS3)


WANT3_BITS = {
    "pos": [[1071693580, 1052634166], [1034412740, 1067265055], [1042003536, 3210282773], [1061655474, 1050836114]],
    "pos_old": [[1071658410, 1052620844], [1042164849, 1066493080], [1046230092, 3208510956],
                [1062047729, 1050258404]],
}


def push_scene():
    s = scenes.spheres(POS2, RAD2, None, gravity=(0.0, 0.0))
    s.substeps = 1
    return s


def hand_push(refresh):
    """refresh=True: the reference (physics.rs:272-286) -- the pushed bodies'
    snapshots are re-taken from their positions, which include body 1's
    earlier correction; False: the GPU's rule, positions at the start of the
    contact pass."""
    m = [mass(r) for r in RAD2]
    p = [x.copy() for x in POS2]
    s = POS2
    # pair (1, 0): an ordinary contact
    ca, cb = correction(s[1], s[0], RAD2[1], RAD2[0], m[1], m[0])
    p[1] = v2(F(p[1][0] + ca[0]), F(p[1][1] + ca[1]))
    p[0] = v2(F(p[0][0] - cb[0]), F(p[0][1] - cb[1]))
    # pair (2, 0): no contact; pair (2, 1): coincident centres
    push = v2(0.01, 0.0)
    base1 = p[1] if refresh else POS2[1]
    base2 = p[2] if refresh else POS2[2]
    p[2] = v2(F(p[2][0] + push[0]), F(p[2][1] + push[1]))
    p[1] = v2(F(p[1][0] - push[0]), F(p[1][1] - push[1]))
    sa = v2(F(F(base2[0] + push[0]) + F(0.0)), F(F(base2[1] + push[1]) + F(0.0)))
    sb = v2(F(F(base1[0] - push[0]) + F(0.0)), F(F(base1[1] - push[1]) + F(0.0)))
    ca, cb = correction(sa, sb, RAD2[2], RAD2[1], m[2], m[1])
    p[2] = v2(F(p[2][0] + ca[0]), F(p[2][1] + ca[1]))
    p[1] = v2(F(p[1][0] - cb[0]), F(p[1][1] - cb[1]))
    return update_objects(p, POS2)


# largest |position difference| between the reference's push-out and the
# GPU's in this scene: body 1's earlier correction moves its refreshed
# snapshot past body 2's, so the reference pushes body 2 the other way
PUSHOUT_DEVIATION = 1.8319036960601807


def three_scene():
    s = scenes.spheres(POS3, RAD3, None, gravity=(0.0, 0.0))
    s.substeps = 1
    return s


def bits(a):
    return np.asarray(a, F).view(np.uint32)


def test_hand_values_match_the_literals_and_depend_on_the_order():
    pos, pold, _ = hand_three()
    assert bits(pos).tolist() == WANT3_BITS["pos"]
    assert bits(pold).tolist() == WANT3_BITS["pos_old"]
    for other in ((2, 1, 0), (1, 0, 2), (0, 2, 1)):
        assert not np.array_equal(bits(hand_three(other)[0])[3], bits(pos)[3]), other


def test_oracle_reproduces_the_three_contact_order():
    pos, pold, vel = hand_three()
    o = oracle.OracleWorld(three_scene(), 32)
    assert o.step(DT, 1) == 0
    got = o.bodies()
    assert np.array_equal(bits(got["pos"].astype(F)), bits(pos))
    assert np.array_equal(bits(got["pos_old"].astype(F)), bits(pold))
    assert np.array_equal(bits(got["vel"].astype(F)), bits(vel))
    assert o.contacts == 3


def test_oracle_reproduces_the_reference_push_out():
    want = hand_push(refresh=True)
    o = oracle.OracleWorld(push_scene(), 32)
    assert o.step(DT, 1) == 0
    got = o.bodies()
    for k, w in zip(("pos", "pos_old", "vel"), want):
        assert np.array_equal(bits(got[k].astype(F)), bits(w)), k
    assert o.pushouts == 1


def test_push_out_deviation_is_the_stated_amount():
    ref, gpu = hand_push(refresh=True)[0], hand_push(refresh=False)[0]
    dev = float(np.abs(ref.astype(np.float64) - gpu.astype(np.float64)).max())
    assert dev == pytest.approx(PUSHOUT_DEVIATION, rel=1e-6)


@pytest.mark.gpu
def test_gpu_reproduces_the_three_contact_order():
    pos, pold, vel = hand_three()
    with native.World(three_scene()) as w:
        w.step(DT)
        got = w.read_bodies()
        assert w.contact_count()[0] == 3
    assert np.array_equal(bits(got["pos"]), bits(pos))
    assert np.array_equal(bits(got["pos_old"]), bits(pold))
    assert np.array_equal(bits(got["vel"]), bits(vel))


@pytest.mark.gpu
def test_gpu_push_out_follows_its_documented_rule():
    want = hand_push(refresh=False)
    with native.World(push_scene()) as w:
        w.step(DT)
        got = w.read_bodies()
        assert w.pushout_count() == 1
    for k, wv in zip(("pos", "pos_old", "vel"), want):
        assert np.array_equal(bits(got[k]), bits(wv)), k
