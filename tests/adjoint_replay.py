"""Reverse-mode derivative of a traced oracle rollout, by replay.

Test infrastructure for the differentiable rollout.  The f32 oracle records
the state at the start of every substep and the contacts that substep
resolved (oracle_world_trace).  Walking the substeps backwards, each one is
re-evaluated in float64 with torch autograd at its recorded state, with its
recorded contact set, and its vector-Jacobian product carries the adjoints
(position, position_old, snapshot, calculated_velocity) one substep back.
The result is the derivative of the f32 trajectory the GPU follows bit for
bit -- same contact sets, same clamps -- evaluated in float64, so it pins
the GPU adjoint without the f32/f64 trajectory drift that a finite
difference of the f64 oracle carries over long horizons.

One substep of a world of single-sphere bodies (blobs/src/physics.rs:397-422):
gravity and springs at the start-of-substep positions and velocities
(springs.rs:25-47, with the `f32 - Vec2` broadcast of springs.rs:41), the
mass-ratio contact correction on the collider snapshots (physics.rs:241-317),
update_objects with the velocity request and the dt / old_dt ratio of the
first dynamic body (physics.rs:323-367), then the wall clamp.
"""
import numpy as np
import torch


def _mass(scene):
    # the lone sphere's mass (0 + 2r) + 2r, exact in f32 (rigid_body.rs:96-128)
    r = scene.col_radius.astype(np.float32)
    return ((np.float32(0.0) + np.float32(2.0) * r) + np.float32(2.0) * r).astype(np.float64)


def _substep(sc, x, v0, k, pairs, first, ratio_first):
    """One substep in float64: inputs p, po, s, v (tensors), outputs p', po', s', v'."""
    p, po, s, v = x
    h = sc["h"]
    dyn = sc["dyn"]
    acc = sc["grav"]
    if sc["n_springs"]:
        ia, ib = sc["spr_a"], sc["spr_b"]
        d = p[ib] - p[ia]
        dist = torch.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1])
        e = d / dist[:, None]
        rv = v[ia] - v[ib]
        q = (rv * e).sum(1)
        fm = (k * (dist - sc["rest"]))[:, None] - e * (sc["c"] * q)[:, None]
        f = e * fm
        fa = torch.where(dyn[ia, None], f / sc["m"][ia, None], torch.zeros_like(f))
        fb = torch.where(dyn[ib, None], -f / sc["m"][ib, None], torch.zeros_like(f))
        acc = acc.index_add(0, ia, fa).index_add(0, ib, fb)
    pc = p
    hi, lo, pushed = pairs
    if len(hi):
        assert not pushed.any(), "push-out contacts are not differentiated"
        hi_t, lo_t = torch.from_numpy(hi), torch.from_numpy(lo)
        ax = s[hi_t] - s[lo_t]
        dl = torch.sqrt(ax[:, 0] * ax[:, 0] + ax[:, 1] * ax[:, 1])
        n = ax / dl[:, None]
        delta = (sc["r"][hi_t] + sc["r"][lo_t]) - dl
        m_hi, m_lo = sc["m"][hi_t], sc["m"][lo_t]
        rho = 1.0 - m_hi / (m_hi + m_lo)
        pc = pc.index_add(0, hi_t, n * (rho * delta)[:, None])
        pc = pc.index_add(0, lo_t, -n * ((1.0 - rho) * delta)[:, None])
    po_eff = po
    if first:
        po_eff = torch.where(sc["vreq_set"][:, None], pc - v0 * h, po)
    ratio = torch.ones(p.shape[0], 1, dtype=torch.float64)
    if sc["first_dyn"] >= 0:
        ratio[sc["first_dyn"], 0] = ratio_first
    disp = (pc - po_eff) * ratio
    pnew = pc + (disp + acc * h * h)
    pnew = torch.where(dyn[:, None], pnew, pc)
    v_new = torch.where(dyn[:, None], disp / h, torch.zeros_like(disp))
    s_new = pnew
    if sc["box"] is not None:
        p_new = torch.minimum(torch.maximum(pnew, sc["box_lo"]), sc["box_hi"])
    else:
        p_new = pnew
    return p_new, pc, s_new, v_new


def _context(scene, dt):
    n = scene.n_bodies
    dyn = scene.body_type != 1
    first_dyn = int(np.flatnonzero(dyn)[0]) if dyn.any() else -1
    r = torch.from_numpy(scene.col_radius.astype(np.float64))
    sc = {
        "h": float(np.float32(np.float32(dt) / np.float32(scene.substeps))),
        "dyn": torch.from_numpy(dyn),
        "first_dyn": first_dyn,
        "m": torch.from_numpy(_mass(scene)),
        "r": r,
        "grav": torch.from_numpy(np.where(dyn[:, None], scene.gravity.astype(np.float64)[None, :]
                                          * scene.gravity_mod.astype(np.float64)[:, None], 0.0)),
        "n_springs": scene.n_springs,
        "spr_a": torch.from_numpy(scene.spr_a.astype(np.int64)),
        "spr_b": torch.from_numpy(scene.spr_b.astype(np.int64)),
        "rest": torch.from_numpy(scene.spr_rest.astype(np.float64)),
        "c": torch.from_numpy(scene.spr_c.astype(np.float64)),
        "vreq_set": torch.from_numpy(scene.vreq_set.astype(bool)),
        "box": scene.world_box,
    }
    if scene.world_box is not None:
        b = scene.world_box[0].astype(np.float32)
        rr = scene.col_radius.astype(np.float32)
        # lo + r and hi - r in f32, as the clamp bounds are formed
        sc["box_lo"] = torch.from_numpy(np.stack([b[0] + rr, b[1] + rr], 1).astype(np.float64))
        sc["box_hi"] = torch.from_numpy(np.stack([b[2] - rr, b[3] - rr], 1).astype(np.float64))
    return sc


def replay_gradients(scene, trace, final_pos, dl_dpos, dt, old_dt=1.0, vreq_pending=True):
    """dL/d(velocity requests) (n, 2) and dL/d(spring stiffness) of a traced
    rollout of one world (single-sphere bodies), given dL/d(final positions).
    Also returns, per state component, the largest difference between a
    replayed substep and the next recorded state (the replay's own check
    against the oracle: f32 rounding, amplified by 1 / dt for velocities)."""
    assert scene.single_collider()
    sc = _context(scene, dt)
    h = sc["h"]
    ratio_first = float(np.float32(np.float32(h) / np.float32(old_dt)))
    v0 = torch.from_numpy(scene.vreq.astype(np.float64)).requires_grad_(True)
    k = torch.from_numpy(scene.spr_k.astype(np.float64)).requires_grad_(True)
    T = len(trace)
    z = lambda: torch.zeros(scene.n_bodies, 2, dtype=torch.float64)
    lam = [torch.from_numpy(np.asarray(dl_dpos, np.float64).copy()), z(), z(), z()]
    gv = np.zeros((scene.n_bodies, 2))
    gk = np.zeros(scene.n_springs)
    worst = {"pos": 0.0, "pos_old": 0.0, "snap": 0.0, "vel": 0.0}
    for t in range(T - 1, -1, -1):
        st = trace[t]
        x = [torch.from_numpy(st[key].copy()).requires_grad_(True) for key in ("pos", "pos_old", "snap", "vel")]
        out = _substep(sc, x, v0, k, (st["hi"], st["lo"], st["pushed"]), t == 0 and vreq_pending,
                       ratio_first if t == 0 else 1.0)
        nxt = final_pos if t == T - 1 else trace[t + 1]["pos"]
        worst["pos"] = max(worst["pos"], float(np.abs(out[0].detach().numpy() - nxt).max()))
        if t < T - 1:
            for key, o in zip(("pos_old", "snap", "vel"), out[1:]):
                worst[key] = max(worst[key], float(np.abs(o.detach().numpy() - trace[t + 1][key]).max()))
        ins = x + [v0, k]
        grads = torch.autograd.grad(out, ins, grad_outputs=lam, allow_unused=True)
        lam = [g if g is not None else torch.zeros_like(i) for g, i in zip(grads[:4], x)]
        if grads[4] is not None:
            gv += grads[4].numpy()
        if grads[5] is not None:
            gk += grads[5].numpy()
    return gv, gk, worst


def tangent_fd(scene, trace, dl_dpos, dt, param, old_dt=1.0, vreq_pending=True, h=1e-4):
    """dL/d(one parameter) by f64 central finite differences chained along a
    traced rollout: the tangent of the state is carried forward substep by
    substep, each substep's directional derivative taken by central
    differences of the f64 substep map at the recorded
    state with the recorded contact set.  No autograd and no adjoint: an
    independent check of the same derivative (that of the f32 trajectory the
    GPU follows).  param = ("v", body, axis) or ("k", spring).  The stencil
    is fourth order, (8 (F(+e) - F(-e)) - (F(+2e) - F(-2e))) / 12e, with the
    step e = h / (largest tangent component) so that the state moves by h.
    Returns (gradient, branch_changed): the second is True when the wall
    clamp of some body differed between the stencil's points in a substep
    (the derivative is then not defined there and the sample is discarded)."""
    assert scene.single_collider()
    sc = _context(scene, dt)
    hs = sc["h"]
    ratio_first = float(np.float32(np.float32(hs) / np.float32(old_dt)))
    n = scene.n_bodies
    v0 = torch.from_numpy(scene.vreq.astype(np.float64))
    k = torch.from_numpy(scene.spr_k.astype(np.float64))
    dv0 = torch.zeros_like(v0)
    dk = torch.zeros_like(k)
    if param[0] == "v":
        dv0[param[1], param[2]] = 1.0
    else:
        dk[param[1]] = 1.0
    tan = [torch.zeros(n, 2, dtype=torch.float64) for _ in range(4)]
    changed = False
    with torch.no_grad():
        for t in range(len(trace)):
            st = trace[t]
            x = [torch.from_numpy(st[key].copy()) for key in ("pos", "pos_old", "snap", "vel")]
            first = t == 0 and vreq_pending
            dpar_v = dv0 if first else torch.zeros_like(dv0)
            s = max(1.0, max(float(tt.abs().max()) for tt in tan), float(dpar_v.abs().max()), float(dk.abs().max()))
            e = h / s
            pairs = (st["hi"], st["lo"], st["pushed"])
            rf = ratio_first if t == 0 else 1.0
            ev = {}
            for j in (-2, -1, 1, 2):
                ev[j] = _substep(sc, [xi + (j * e) * ti for xi, ti in zip(x, tan)], v0 + (j * e) * dpar_v,
                                 k + (j * e) * dk, pairs, first, rf)
            if sc["box"] is not None:
                masks = [ev[j][0] != ev[j][2] for j in (-2, -1, 1, 2)]
                changed = changed or any(bool((mk != masks[0]).any()) for mk in masks[1:])
            # fourth-order central stencil
            tan = [(8.0 * (a1 - m1) - (a2 - m2)) / (12.0 * e)
                   for a1, m1, a2, m2 in zip(ev[1], ev[-1], ev[2], ev[-2])]
    g = float((torch.from_numpy(np.asarray(dl_dpos, np.float64)) * tan[0]).sum())
    return g, changed
