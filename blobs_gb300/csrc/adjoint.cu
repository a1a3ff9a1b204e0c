// adjoint.cu -- reverse-mode derivative of one single-sphere substep
// (physics.rs:397-422 for worlds of single spheres with springs and walls),
// the building block of blobs_world_backward.
//
// Forward map of a substep for a dynamic body (state at its start: position
// p, position_old po, snapshot s, calculated_velocity v):
//   p_c   = p + sum_contacts corr(s_self, s_other)         (physics.rs:291-300)
//   disp  = (p_c - po) * ratio                             (physics.rs:338)
//   a     = g gm + sum_springs F(p, v; k) / m               (springs.rs:25-47)
//   p_new = p_c + (disp + a dt dt);  s' = p_new            (physics.rs:343-344, :360-366)
//   p'    = clamp(p_new);  po' = p_c;  v' = disp / dt
// and on the rollout's first substep a velocity request replaces po by
// p_c - v0 dt (physics.rs:334-336), so disp = v0 dt ratio.  Push-out
// contacts are discrete events and are not differentiated.
//
// Three kernels per substep, in order:
//   k_adj_body    per body: Verlet, clamp mask, velocity request -> the
//                 adjoints of p_c and a, the outgoing adjoint of po
//   k_adj_springs per spring: Jacobians of the (quirky) spring force ->
//                 the adjoints of the spring's d = pb - pa and rv = va - vb,
//                 and dL/dk
//   k_adj_gather  per body: its recorded contacts (the Jacobian of the
//                 mass-ratio correction, each pair evaluated from both
//                 sides) -> the adjoint of its snapshot; its springs ->
//                 the adjoints of its position and velocity
// Every sum runs in a fixed order (ascending partner id, ascending spring
// index), so the gradients are deterministic: no float atomics.
#include "device.cuh"
#include "kernels.h"

namespace blobs {

__global__ void __launch_bounds__(256) k_adj_body(WorldDev w, AdjointSubstep a) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= w.n_bodies) return;
  const uint8_t fl = w.bflags[b];
  const float dt = a.dt;
  // clamp mask of the wall extension: the derivative passes where the body
  // was not clamped
  const WorldParam wp = w.wparam[w.n_worlds > 1 ? w.body_world[b] : 0u];
  const float2 s1 = a.s_t1[b];
  float2 mask = v2(1.0f, 1.0f);
  if (wp.has_box) {
    const float br = w.bound_r[b];
    mask.x = (s1.x > wp.box_lo_x + br && s1.x < wp.box_hi_x - br) ? 1.0f : 0.0f;
    mask.y = (s1.y > wp.box_lo_y + br && s1.y < wp.box_hi_y - br) ? 1.0f : 0.0f;
  }
  const float2 lp1 = a.lp_in[b], lpo1 = a.lpo_in[b], ls1 = a.ls_in[b], lv1 = a.lv_in[b];
  const float2 lpnew = v2(ls1.x + mask.x * lp1.x, ls1.y + mask.y * lp1.y);
  float2 lpc, la = v2(0.0f, 0.0f), lpo = v2(0.0f, 0.0f);
  if (fl & BF_STATIC) {
    // static: p_new = p_c, po' = p_c, v' = 0
    lpc = add(lpnew, lpo1);
  } else {
    const float ratio = (a.first_substep && (fl & BF_FIRST_DYN)) ? a.ratio_first : 1.0f;
    const float2 ldisp = add(lpnew, mul(lv1, 1.0f / dt));
    la = mul(lpnew, dt * dt);
    lpc = add(lpnew, lpo1);
    if (a.first_substep && a.vreq_pending && (fl & BF_VREQ)) {
      // disp = (p_c - (p_c - v0 dt)) ratio: no dependence on p_c or po
      const float2 g = mul(ldisp, dt * ratio);
      a.lv0[b] = add(a.lv0[b], g);
    } else {
      lpc = add(lpc, mul(ldisp, ratio));
      lpo = mul(ldisp, -ratio);
    }
  }
  a.lpc[b] = lpc;
  a.la[b] = la;
  a.lpo_out[b] = lpo;
}

__global__ void __launch_bounds__(256) k_adj_springs(WorldDev w, AdjointSubstep a) {
  const uint32_t sidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (sidx >= w.n_springs) return;
  a.spr_terms[sidx] = make_float4(0.f, 0.f, 0.f, 0.f);
  const uint32_t ia = w.spr_a[sidx], ib = w.spr_b[sidx];
  const bool sa_static = (w.bflags[ia] & BF_STATIC) != 0, sb_static = (w.bflags[ib] & BF_STATIC) != 0;
  // force adjoint: a_a += F / m_a, a_b += -F / m_b (static bodies take no force)
  const float2 laa = a.la[ia], lab = a.la[ib];
  const float ma = w.mass[ia], mb = w.mass[ib];
  float mux = 0.0f, muy = 0.0f;
  if (!sa_static) mux += laa.x / ma, muy += laa.y / ma;
  if (!sb_static) mux -= lab.x / mb, muy -= lab.y / mb;
  if (mux == 0.0f && muy == 0.0f) return;
  const float2 pa = a.p_t[ia], pb = a.p_t[ib];
  const float dx = pb.x - pa.x, dy = pb.y - pa.y;
  const float dist = sqrtf(dx * dx + dy * dy);
  if (!(dist > 0.0f)) return;
  const float ex = dx / dist, ey = dy / dist;
  const float k = w.spr_k[sidx], c = w.spr_c[sidx], L = w.spr_rest[sidx];
  float rvx = 0.0f, rvy = 0.0f;
  if (a.v_t) {
    const float2 va = a.v_t[ia], vb = a.v_t[ib];
    rvx = va.x - vb.x;
    rvy = va.y - vb.y;
  }
  const float q = rvx * ex + rvy * ey;
  // P = (I - e e^T) / dist = d e / d d
  const float inv = 1.0f / dist;
  const float pxx = (1.0f - ex * ex) * inv, pyy = (1.0f - ey * ey) * inv, pxy = -ex * ey * inv;
  // dq/dd = rv^T P
  const float dqx = rvx * pxx + rvy * pxy, dqy = rvx * pxy + rvy * pyy;
  const float el = k * (dist - L);
  // F_i = k (dist - L) e_i - c q e_i^2   (the f32 - Vec2 broadcast, springs.rs:41)
  // dF_i/dd_j = k e_j e_i + k (dist - L) P_ij - c (e_i^2 dq_j + 2 q e_i P_ij)
  const float fxx = k * ex * ex + el * pxx - c * (ex * ex * dqx + 2.0f * q * ex * pxx);
  const float fxy = k * ey * ex + el * pxy - c * (ex * ex * dqy + 2.0f * q * ex * pxy);
  const float fyx = k * ex * ey + el * pxy - c * (ey * ey * dqx + 2.0f * q * ey * pxy);
  const float fyy = k * ey * ey + el * pyy - c * (ey * ey * dqy + 2.0f * q * ey * pyy);
  const float ldx = fxx * mux + fyx * muy, ldy = fxy * mux + fyy * muy;
  // dF_i/drv_j = -c e_i^2 e_j
  const float lrvx = -c * (ex * ex * ex * mux + ey * ey * ex * muy);
  const float lrvy = -c * (ex * ex * ey * mux + ey * ey * ey * muy);
  // dF_i/dk = (dist - L) e_i
  a.lk[sidx] += (dist - L) * (ex * mux + ey * muy);
  // d = pb - pa, rv = va - vb: k_adj_gather adds +-these at both ends
  a.spr_terms[sidx] = make_float4(ldx, ldy, lrvx, lrvy);
}

__global__ void __launch_bounds__(256) k_adj_gather(WorldDev w, AdjointSubstep a) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= w.n_bodies) return;
  // contacts: p_c(hi) += rho d(n) ... on s_hi - s_lo, evaluated from this body's side
  float2 ls = v2(0.0f, 0.0f);
  const uint32_t nrec = min(a.rec_n[c], REC_CAP);
  const float2 sc = a.s_t[c];
  const float rc = w.col_radius[c], mc = w.mass[c];
  for (uint32_t e = 0; e < nrec; ++e) {
    const uint32_t rec = a.rec_list[(size_t)e * w.n_bodies + c];
    if (rec & 0x80000000u) continue;  // push-out: not differentiated
    const uint32_t o = rec;
    if (o >= w.n_bodies || o == c) continue;
    const bool hi = c > o;
    const uint32_t ia = hi ? c : o, ib = hi ? o : c;
    const float2 so = a.s_t[o];
    const float2 sa = hi ? sc : so, sb = hi ? so : sc;
    const float ax = sa.x - sb.x, ay = sa.y - sb.y;
    const float d = sqrtf(ax * ax + ay * ay);
    if (!(d > 0.0f)) continue;
    const float nx = ax / d, ny = ay / d;
    const float R = rc + w.col_radius[o];
    const float mo = w.mass[o];
    const float ma = hi ? mc : mo, mb = hi ? mo : mc;
    const float rho = 1.0f - ma / (ma + mb);
    // corr_a = rho * delta * n, corr_b = -(1 - rho) * delta * n with
    // delta n = R axis / d - axis; d(delta n)/d axis = J = (R/d)(I - n n^T) - I, symmetric
    const float2 la_ = a.lpc[ia], lb_ = a.lpc[ib];
    const float ux = rho * la_.x - (1.0f - rho) * lb_.x, uy = rho * la_.y - (1.0f - rho) * lb_.y;
    const float q = R / d;
    const float jxx = q * (1.0f - nx * nx) - 1.0f, jyy = q * (1.0f - ny * ny) - 1.0f, jxy = -q * nx * ny;
    const float gx = jxx * ux + jxy * uy, gy = jxy * ux + jyy * uy;
    ls = hi ? v2(ls.x + gx, ls.y + gy) : v2(ls.x - gx, ls.y - gy);
  }
  a.ls_out[c] = ls;
  // springs, ascending spring index: p_c = p + corrections(s), so the
  // position adjoint is lpc plus the spring terms
  float2 lp = a.lpc[c], lv = v2(0.0f, 0.0f);
  if (w.n_springs) {
    const uint32_t q0 = w.body_spr_start[c], q1 = w.body_spr_start[c + 1];
    for (uint32_t qq = q0; qq < q1; ++qq) {
      const uint32_t e = w.body_spr[qq];
      const float4 t = a.spr_terms[e >> 1];
      if (e & 1u) {  // endpoint b: +d, -rv
        lp = v2(lp.x + t.x, lp.y + t.y);
        lv = v2(lv.x - t.z, lv.y - t.w);
      } else {       // endpoint a: -d, +rv
        lp = v2(lp.x - t.x, lp.y - t.y);
        lv = v2(lv.x + t.z, lv.y + t.w);
      }
    }
  }
  a.lp_out[c] = lp;
  a.lv_out[c] = lv;
}

void launch_adjoint_substep(const WorldDev& w, const AdjointSubstep& a, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_adj_body<<<(w.n_bodies + 255u) / 256u, 256, 0, st>>>(w, a);
  if (w.n_springs) k_adj_springs<<<(w.n_springs + 255u) / 256u, 256, 0, st>>>(w, a);
  k_adj_gather<<<(w.n_bodies + 255u) / 256u, 256, 0, st>>>(w, a);
}

}  // namespace blobs
