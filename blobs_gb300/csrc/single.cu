// single.cu -- the single-sphere path: every body owns exactly one collider
// at offset zero with default groups and no sensor, and there are no fixed
// joints (sparse and dense sphere worlds, uneven batches, the gradient batch).
//
// Body state lives in "storage order", re-sorted into cell order once per
// step, so that a warp's bodies are spatial neighbours:
//   A[slot] = (snapshot x, snapshot y, radius, arena id bits)
//   B[slot] = (position x, y, position_old x, y)
//   V[slot] = calculated_velocity (or, without springs, the last
//             substep's displacement; the division by dt happens on read)
// A, B, V are double-buffered per substep.  Per substep:
//   k_permute      (first substep of a step) storage -> this substep's cell
//                  order; the permuted A is then also the candidate array
//   k_scatter_cand (other substeps) a cell-order copy of A for the
//                  candidate search (16 B per body instead of the record)
//   k_step_single  per slot: gravity + springs, contacts over the 3x3 cells
//                  applied in the reference's pair order, Verlet
//                  integration, constraints, next cell key / rank
// Compiled with --fmad=false (see device.cuh).
#include "device.cuh"
#include "kernels.h"

namespace blobs {

namespace {

__device__ __forceinline__ uint32_t rec_flags(float4 c) { return __float_as_uint(c.w) & 0xffu; }
__device__ __forceinline__ uint32_t rec_world(float4 c) { return __float_as_uint(c.w) >> 8; }

// The cell-order positions of the 3 rows of 3 cells around cell `key`: up to
// six contiguous segments (a row splits in two where the torus wraps).
struct Segments {
  uint32_t s[6], l[6];
};

__device__ __forceinline__ Segments segments(const WorldDev& w, const WorldParam& wp, uint32_t key) {
  Segments g;
  const uint32_t wm = (1u << wp.log2w) - 1u, hm = (1u << wp.log2h) - 1u;
  const uint32_t local = key - wp.cell_base;
  const uint32_t ix = local & wm, iy = local >> wp.log2w;
  const uint32_t x0 = (ix - 1u) & wm, x2 = (ix + 1u) & wm;
  const uint32_t n = w.n_cols;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const uint32_t row = wp.cell_base + (((iy + (uint32_t)(r - 1)) & hm) << wp.log2w);
    uint32_t a0, a1, b0, b1;
    if (x0 < x2) {
      a0 = w.cell_start[row + x0];
      a1 = w.cell_start[row + x2 + 1u];
      b0 = b1 = 0u;
    } else {
      a0 = w.cell_start[row + x0];
      a1 = w.cell_start[row + wm + 1u];
      b0 = w.cell_start[row];
      b1 = w.cell_start[row + x2 + 1u];
    }
    a1 = min(a1, n);
    b1 = min(b1, n);
    g.s[2 * r] = a0;
    g.l[2 * r] = a1 > a0 ? a1 - a0 : 0u;
    g.s[2 * r + 1] = b0;
    g.l[2 * r + 1] = b1 > b0 ? b1 - b0 : 0u;
  }
  return g;
}

// Position of the t-th candidate of the segments (t < total).
__device__ __forceinline__ uint32_t slot_of(const Segments& g, uint32_t t) {
  uint32_t q = g.s[5] + t;
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const uint32_t lo = acc;
    acc += g.l[k];
    if (t >= lo && t < acc) q = g.s[k] + (t - lo);
  }
  if (t >= acc) q = g.s[5] + (t - acc);
  return q;
}

// Near test of four consecutive candidate positions [q, q + 4) clipped to
// `en`, loads issued together for memory-level parallelism.

__device__ __forceinline__ void near_range(const float4* __restrict__ C, float2 s, float r, uint32_t self,
                                           uint32_t st, uint32_t en, uint32_t& t, unsigned long long& near) {
  for (uint32_t q = st; q < en; q += 4u, t += 4u) {
    const float4 far = make_float4(3.0e38f, 3.0e38f, 0.0f, 0.0f);
    const float4 o0 = C[q];
    const float4 o1 = q + 1u < en ? C[q + 1u] : far;
    const float4 o2 = q + 2u < en ? C[q + 2u] : far;
    const float4 o3 = q + 3u < en ? C[q + 3u] : far;
    uint32_t m = 0u;
    if (near_pair(s.x - o0.x, s.y - o0.y, r + o0.z) && __float_as_uint(o0.w) != self) m |= 1u;
    if (near_pair(s.x - o1.x, s.y - o1.y, r + o1.z) && __float_as_uint(o1.w) != self) m |= 2u;
    if (near_pair(s.x - o2.x, s.y - o2.y, r + o2.z) && __float_as_uint(o2.w) != self) m |= 4u;
    if (near_pair(s.x - o3.x, s.y - o3.y, r + o3.z) && __float_as_uint(o3.w) != self) m |= 8u;
    if (m) near |= (unsigned long long)m << t;
  }
}

struct SinglePair {
  float2 corr;
  float2 push;
  bool pushed;
};

// The increment to body c's position from its contact with body c2, in the
// reference's terms (a = the higher arena index).  Returns false if the pair
// is not in contact.  The push-out branch (physics.rs:272-286) uses the
// positions at the start of the contact pass: p, or with LOAD_P the one
// loaded from body c's slot jc.
template <bool LOAD_P = false>
__device__ __forceinline__ bool single_pair(const WorldDev& w, const SingleArgs& a, uint32_t c, float2 p, float2 s,
                                            float r, float m, uint32_t c2, float2 s2, float r2, float m2,
                                            SinglePair& out, uint32_t jc = 0u) {
  const float dx = s.x - s2.x, dy = s.y - s2.y;
  const float mind = r + r2;
  float d = sqrtf((dx * dx) + (dy * dy));
  if (!(d < mind)) return false;
  const bool hi = c > c2;
  float2 axis = hi ? v2(dx, dy) : v2(-dx, -dy);
  out.pushed = false;
  out.push = v2(0.0f, 0.0f);
  if (d < 1e-6f) {
    if (LOAD_P) {
      const float4 b1 = a.b_in[jc];
      p = v2(b1.x, b1.y);
    }
    const float4 b2 = a.b_in[w.where[c2]];
    const float2 p2 = v2(b2.x, b2.y);
    const float2 pa = add(hi ? p : p2, v2(0.01f, 0.0f));
    const float2 pb = sub(hi ? p2 : p, v2(0.01f, 0.0f));
    axis = sub(add(pa, v2(0.0f, 0.0f)), add(pb, v2(0.0f, 0.0f)));
    d = len2(axis);
    out.pushed = true;
    out.push = hi ? v2(0.01f, 0.0f) : v2(-0.01f, -0.0f);
  }
  const float2 n = divs(axis, d);
  if (n.x != n.x || n.y != n.y) atomicOr(w.status, ST_NAN);
  const float delta = mind - d;
  const float ma = hi ? m : m2, mb = hi ? m2 : m;
  const float ratio = 1.0f - ma / (ma + mb);
  if (hi) {
    out.corr = mul(n, ratio * delta);
  } else {
    const float2 t = mul(n, (1.0f - ratio) * delta);
    out.corr = v2(-t.x, -t.y);
  }
  return true;
}

// Record a contact of body c (its partner, in the order applied) for the
// adjoint pass.
__device__ __forceinline__ void record_contact(const WorldDev& w, const SingleArgs& a, uint32_t c, uint32_t other,
                                               bool pushed, uint32_t& nrec) {
  if (nrec < REC_CAP) a.rec_list[(size_t)nrec * w.n_bodies + c] = other | (pushed ? 0x80000000u : 0u);
  ++nrec;
}

// Collision event of the pair (c, lo), c > lo: velocities from the V buffer
// (calculated_velocity while events are on) at both bodies' storage slots.
__device__ __forceinline__ void single_event(const WorldDev& w, const SingleArgs& a, uint32_t c, uint32_t j,
                                             uint32_t lo) {
  const uint32_t jl = w.where[lo];
  if (jl >= w.n_bodies) {
    atomicOr(w.status, ST_BAD_INDEX);
    return;
  }
  record_event(w, c, lo, a.v_in[j], a.v_in[jl]);
}

__device__ __forceinline__ void count_warp(const WorldDev& w, uint32_t ncontacts, uint32_t npush, bool deferred) {
  uint32_t t = ncontacts, p = npush;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_xor_sync(0xffffffffu, t, o);
    p += __shfl_xor_sync(0xffffffffu, p, o);
  }
  const uint32_t nw = __popc(__ballot_sync(0xffffffffu, deferred));
  if ((threadIdx.x & 31u) == 0u) {
    const uint32_t bin = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) & (COUNTER_BINS - 1);
    if (t) {
      atomicAdd(w.contacts_total + bin, (unsigned long long)t);
      atomicAdd(w.contacts_sub + bin, t);
    }
    if (p) atomicAdd(w.pushouts_total + bin, (unsigned long long)p);
    if (nw) {
      atomicAdd(w.defer_total + bin, (unsigned long long)nw);
      atomicAdd(w.defer_sub + bin, nw);
    }
  }
}

// Mass, gravity_mod, bounding radius, flags and world of the body with
// arena id c.  A uniform world (default collider masses, no static body, one
// gravity_mod, one world) needs no per-body record: the reference's mass of
// a lone sphere is (0 + 2r) + 2r = 4r exactly (rigid_body.rs:96-128 with the
// doubled handle), its bounding radius |0| + r = r.
struct BodyConst {
  float m, gm, br;
  uint32_t flags, world;
};

template <int MODE>  // 0: one world, uniform; 1: one world, per-body record; 2: batched, per-body record
__device__ __forceinline__ BodyConst body_const(const WorldDev& w, const WorldParam& wp0, uint32_t c, float r) {
  BodyConst k;
  if (MODE == 0) {
    k.m = r * 4.0f;
    k.gm = wp0.uniform_gmod;
    k.br = r;
    k.flags = (c == wp0.first_dyn) ? (uint32_t)BF_FIRST_DYN : 0u;
    k.world = 0u;
  } else {
    const float4 rec = w.body_c[c];
    k.m = rec.x;
    k.gm = rec.y;
    k.br = rec.z;
    k.flags = rec_flags(rec);
    k.world = MODE == 2 ? rec_world(rec) : 0u;
  }
  return k;
}

// Exact selection walk over all candidates of the segments, in ascending
// arena id (many candidates, or any layout): O(contacts x candidates).
// HOOKS: the adjoint's contact recording or the event stream may be on.
template <int MODE, bool HOOKS>
__device__ float2 contacts_walk(const WorldDev& w, const SingleArgs& a, const Segments& g, uint32_t j, uint32_t c,
                                float2 p0, float2 s, float r, float m, uint32_t& ncontacts, uint32_t& npush,
                                uint32_t& nrec) {
  const float4* __restrict__ C = a.cand;
  float2 p = p0;
  uint32_t last = 0u;
  bool first = true;
  while (true) {
    uint32_t best = 0xffffffffu;
    float4 bo = make_float4(0.f, 0.f, 0.f, 0.f);
    bool found = false;
    for (int sg = 0; sg < 6; ++sg) {
      const uint32_t q1 = g.s[sg] + g.l[sg];
      for (uint32_t q = g.s[sg]; q < q1; ++q) {
        const float4 o = C[q];
        const uint32_t c2 = __float_as_uint(o.w);
        if (c2 == c || c2 >= w.n_bodies || (!first && c2 <= last) || (found && c2 >= best)) continue;
        const float dx = s.x - o.x, dy = s.y - o.y;
        if (!(sqrtf((dx * dx) + (dy * dy)) < r + o.z)) continue;
        best = c2;
        bo = o;
        found = true;
      }
    }
    if (!found) break;
    const float m2 = (MODE == 0 || a.mass4r) ? bo.z * 4.0f : w.body_c[best].x;
    SinglePair sp;
    single_pair(w, a, c, p0, s, r, m, best, v2(bo.x, bo.y), bo.z, m2, sp);
    if (sp.pushed) p = add(p, sp.push);
    p = add(p, sp.corr);
    if (HOOKS && a.rec_list) record_contact(w, a, c, best, sp.pushed, nrec);
    if (best < c) {
      ++ncontacts;
      npush += sp.pushed ? 1u : 0u;
      if (HOOKS && w.ev_rec) single_event(w, a, c, j, best);
    }
    last = best;
    first = false;
  }
  return p;
}

constexpr int STEP_THREADS = 128;

// Bodies with more near candidates than this take k_step_deferred (the
// per-lane ordered selection is O(near^2)); with phase 2 shared out over
// the warp, more than WARP_NEAR.
constexpr uint32_t DEFER_NEAR = 12;
constexpr uint32_t WARP_NEAR = 32;
constexpr uint32_t DEFER_CAP = 256;    // contacts a deferred body's warp ranks in shared memory
constexpr int DEFER_THREADS = 128;
constexpr uint32_t DEFER_BLOCKS = 152 * 8;

struct DeferWarp {
  uint32_t id[DEFER_CAP];              // partner arena id of each contact found
  float4 corr[DEFER_CAP];              // correction x, y; push-out flag bits
  uint32_t order[DEFER_CAP];           // contacts in ascending partner id
};


}  // namespace

// update_objects (physics.rs:323-367) of one body after its contacts:
// gravity + springs at the start-of-substep state, Verlet, the snapshot, the
// constraints, and the next substep's cell key and rank.  p0 is the position
// at the start of the substep, p the position after the contacts.
template <int MODE>
__device__ __forceinline__ void finish_single(const WorldDev& w, const SingleArgs& a, const WorldParam& wp,
                                              const BodyConst& k, uint32_t j, uint32_t c, float4 av, float4 bv,
                                              float2 p0, float2 p) {
  const float r = av.z;
  // ---- update_objects (physics.rs:323-367) with gravity + springs ----
  const float dt = a.dt;
  float2 po, vel;
  if (k.flags & BF_STATIC) {
    po = p;
    vel = v2(0.0f, 0.0f);
  } else {
    po = v2(bv.z, bv.w);
    uint32_t fl = k.flags;
    if (a.pending && MODE == 0) fl |= rec_flags(w.body_c[c]);
    if (a.pending && (fl & BF_VREQ)) po = sub(p, mul(w.vreq[c], dt));
    const float ratio = (fl & BF_FIRST_DYN) ? a.ratio_first : a.ratio_rest;
    const float2 disp = mul(sub(p, po), ratio);
    float2 acc = a.pending ? w.pend_acc[c] : v2(0.0f, 0.0f);
    acc = add(acc, mul(w.gravity, k.gm));
    if (a.springs) {
      const uint32_t q0 = w.body_spr_start[c], q1 = w.body_spr_start[c + 1];
      for (uint32_t qq = q0; qq < q1; ++qq) {
        const uint32_t e = w.body_spr[qq];
        const uint32_t sidx = e >> 1;
        const uint32_t other = (e & 1u) ? w.spr_a[sidx] : w.spr_b[sidx];
        const uint32_t so = w.where[other];
        const float4 bo = a.b_in[so];
        const float2 po_pos = v2(bo.x, bo.y);
        const float2 po_vel = a.v_in[so];
        const float2 own_vel = a.v_in[j];
        const float2 va = (e & 1u) ? po_vel : own_vel, vb = (e & 1u) ? own_vel : po_vel;
        const float2 pa = (e & 1u) ? po_pos : p0, pb = (e & 1u) ? p0 : po_pos;
        const float2 d = sub(pb, pa);
        const float dist = len2(d);
        const float2 dir = divs(d, dist);
        const float2 rv = sub(va, vb);
        const float2 damping = mul(dir, w.spr_c[sidx] * dot2(rv, dir));
        const float sk = w.spr_k[sidx] * (dist - w.spr_rest[sidx]);
        const float2 fm = v2(sk - damping.x, sk - damping.y);  // springs.rs:41 broadcast
        float2 f = mulv(dir, fm);
        if (e & 1u) f = v2(-f.x, -f.y);
        acc = add(acc, divs(f, k.m));
      }
    }
    po = p;
    p = add(p, add(disp, mul(mul(acc, dt), dt)));
    if (a.rot_dynamic) {
      const float tq = a.pending ? w.pend_torque[c] : 0.0f;
      float avl = w.angvel[c];
      avl = avl + (tq / w.inertia[c]) * dt;
      w.angvel[c] = avl;
      w.rot[c] = w.rot[c] + avl * dt;
    }
    // calculated_velocity = disp / dt (physics.rs:357); without springs or
    // collision events nothing reads it during the step, so the
    // displacement is kept and divided when it is read
    vel = a.v_vel ? divs(disp, dt) : disp;
  }
  const float2 snap = v2(0.0f + p.x, 0.0f + p.y);  // rot(theta) * 0 + p
  for (uint32_t kk = 0; kk < w.n_circles; ++kk) {
    const float2 cc = v2(w.circles[3 * kk], w.circles[3 * kk + 1]);
    const float radius = w.circles[3 * kk + 2];
    const float2 to = sub(p, cc);
    const float dist = len2(to);
    if (dist > radius) p = add(cc, mul(divs(to, dist), radius));
  }
  if (wp.has_box) {
    p.x = fminf(fmaxf(p.x, wp.box_lo_x + k.br), wp.box_hi_x - k.br);
    p.y = fminf(fmaxf(p.y, wp.box_lo_y + k.br), wp.box_hi_y - k.br);
  }
  a.a_out[j] = make_float4(snap.x, snap.y, r, av.w);
  a.b_out[j] = make_float4(p.x, p.y, po.x, po.y);
  if (a.v_vel || a.write_v) a.v_out[j] = vel;
  if (a.do_keys) {
    const uint32_t key = cell_key(wp, snap);
    w.key[j] = key;
    w.rank[j] = atomicAdd(w.cell_count + key, 1u);
  }
}


// Phase 2 per lane (the event, recording and per-body-record variants; at
// most DEFER_NEAR near candidates): the near candidates' ids are gathered
// into this thread's shared-memory slots first
// (independent loads), then the ascending-id selection runs over shared
// memory and only the chosen candidate's record is loaded again.
template <int MODE, bool HOOKS>
__device__ __forceinline__ float2 apply_near_s(const WorldDev& w, const SingleArgs& a, unsigned long long near,
                                               uint32_t s0, uint32_t s1, uint32_t s2, uint32_t t1, uint32_t t2,
                                               uint32_t j, uint32_t c, float2 p0, float2 s, float r, float m,
                                               uint32_t& ncontacts, uint32_t& npush, uint32_t& nrec, uint32_t* ids,
                                               uint32_t* qs, uint32_t* ev_lo, uint32_t& nev) {
  const float4* __restrict__ C = a.cand;
  const uint32_t* __restrict__ Cw = reinterpret_cast<const uint32_t*>(a.cand);
  float2 p = p0;
  uint32_t kk = 0;
  for (unsigned long long mk = near; mk; mk &= mk - 1ull, ++kk) {
    const uint32_t tt = (uint32_t)(__ffsll((long long)mk) - 1);
    const uint32_t q = tt < t1 ? s0 + tt : (tt < t2 ? s1 + (tt - t1) : s2 + (tt - t2));
    ids[kk * STEP_THREADS] = Cw[4u * q + 3u];
    qs[kk * STEP_THREADS] = q;
  }
  uint32_t used = 0u;
  for (uint32_t it = 0; it < kk; ++it) {
    uint32_t best = 0xffffffffu, bi = 0u;
    for (uint32_t i = 0; i < kk; ++i) {
      const uint32_t id = ids[i * STEP_THREADS];
      if (!((used >> i) & 1u) && id < best) {
        best = id;
        bi = i;
      }
    }
    used |= 1u << bi;
    if (best >= w.n_bodies || best == c) continue;
    const float4 bo = C[qs[bi * STEP_THREADS]];
    const float m2 = (MODE == 0 || a.mass4r) ? bo.z * 4.0f : w.body_c[best].x;
    SinglePair sp;
    if (!single_pair(w, a, c, p0, s, r, m, best, v2(bo.x, bo.y), bo.z, m2, sp)) continue;
    if (sp.pushed) p = add(p, sp.push);
    p = add(p, sp.corr);
    if (HOOKS && a.rec_list) record_contact(w, a, c, best, sp.pushed, nrec);
    if (best < c) {
      ++ncontacts;
      npush += sp.pushed ? 1u : 0u;
      if (HOOKS && w.ev_rec) ev_lo[(nev++) * STEP_THREADS] = best;  // appended by the warp afterwards
    }
  }
  return p;
}

// Phase 2 of the plain step in a uniform world, shared out over the warp's
// lanes.  The near candidates of each lane get consecutive slots of the
// warp's PairSlots (the lane's range, in lane order); every lane computes
// the corrections of slots lane, lane + 32, ... with the owner's snapshot,
// radius, mass and id taken by shuffle, and stores each at its rank by
// partner id within the owner's range; then each owner adds its
// corrections in that order, the reference's pair order for this body.
// The exact tests and corrections (a square root and three divisions each)
// thus run on all lanes however unevenly the near candidates fall.  A warp
// with more than PAIR_CAP slots works in rounds of whole ranges.
constexpr uint32_t PAIR_CAP = 128;

struct PairSlots {
  uint32_t id[PAIR_CAP];  // partner arena id
  uint32_t q[PAIR_CAP];   // partner's position in the candidate array
  float cx[PAIR_CAP];     // correction, at its rank in the owner's range
  float cy[PAIR_CAP];
  uint8_t fl[PAIR_CAP];   // at the rank: 1 contact, 2 pushed out, 4 partner id below the owner's
  uint8_t own[PAIR_CAP];  // owner lane
};

// Correction of slot e for its owner (whose values the caller shuffled in),
// stored at the slot's rank in the owner's range [o0, o0 + okk).
template <int MODE>
__device__ __forceinline__ void shared_pair(const WorldDev& w, const SingleArgs& a, PairSlots& S, uint32_t e,
                                            uint32_t jown, float2 so, float ro, float mo, uint32_t co, uint32_t o0,
                                            uint32_t okk) {
  const uint32_t id = S.id[e];
  // rank in the owner's range (ties, which distinct bodies never make,
  // broken by slot so that the ranks stay a permutation)
  uint32_t rank = 0;
  for (uint32_t i = 0; i < okk; ++i) {
    const uint32_t idi = S.id[o0 + i];
    rank += (idi < id || (idi == id && o0 + i < e)) ? 1u : 0u;
  }
  uint32_t f = 0u;
  SinglePair sp;
  sp.corr = v2(0.0f, 0.0f);
  if (id < w.n_bodies && id != co) {
    const float4 bo = a.cand[S.q[e]];
    const float m2 = (MODE == 0 || a.mass4r) ? bo.z * 4.0f : w.body_c[id].x;
    if (single_pair<true>(w, a, co, v2(0.0f, 0.0f), so, ro, mo, id, v2(bo.x, bo.y), bo.z, m2, sp, jown))
      f = 1u | (sp.pushed ? 2u : 0u) | (id < co ? 4u : 0u);
  }
  const uint32_t at = o0 + min(rank, okk - 1u);
  S.cx[at] = sp.corr.x;
  S.cy[at] = sp.corr.y;
  S.fl[at] = (uint8_t)f;
}

// Every lane of the warp calls this; a lane with no near candidates passes
// near = 0 and gets p back.  jbase is the slot of lane 0.
template <int MODE>
__device__ __forceinline__ float2 apply_near_warp(const WorldDev& w, const SingleArgs& a, PairSlots& S,
                                                  uint32_t lane, uint32_t jbase, unsigned long long near,
                                                  uint32_t s0, uint32_t s1, uint32_t s2, uint32_t t1, uint32_t t2,
                                                  uint32_t c, float2 s, float r, float m, float2 p,
                                                  uint32_t& ncontacts, uint32_t& npush) {
  const uint32_t* __restrict__ Cw = reinterpret_cast<const uint32_t*>(a.cand);
  const uint32_t kk = (uint32_t)__popcll(near);
  uint32_t incl = kk;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  const uint32_t off = incl - kk;
  for (uint32_t base = 0; base < total;) {
    // this round: the ranges that lie wholly in [base, base + PAIR_CAP)
    const bool mine = kk > 0u && off >= base && off + kk <= base + PAIR_CAP;
    uint32_t end = mine ? off + kk : base;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) end = max(end, __shfl_xor_sync(0xffffffffu, end, o));
    const uint32_t cnt = end - base, r0 = off - base;
    if (mine) {
      uint32_t e = r0;
      for (unsigned long long mk = near; mk; mk &= mk - 1ull, ++e) {
        const uint32_t tt = (uint32_t)(__ffsll((long long)mk) - 1);
        const uint32_t q = tt < t1 ? s0 + tt : (tt < t2 ? s1 + (tt - t1) : s2 + (tt - t2));
        S.id[e] = Cw[4u * q + 3u];
        S.q[e] = q;
        S.own[e] = (uint8_t)lane;
      }
    }
    __syncwarp();
    for (uint32_t e0 = 0; e0 < cnt; e0 += 32u) {
      const uint32_t e = e0 + lane;
      const uint32_t o = e < cnt ? (uint32_t)S.own[e] : lane;
      const float2 so = v2(__shfl_sync(0xffffffffu, s.x, o), __shfl_sync(0xffffffffu, s.y, o));
      const float ro = __shfl_sync(0xffffffffu, r, o), mo = __shfl_sync(0xffffffffu, m, o);
      const uint32_t co = __shfl_sync(0xffffffffu, c, o);
      const uint32_t o0 = __shfl_sync(0xffffffffu, r0, o), okk = __shfl_sync(0xffffffffu, kk, o);
      if (e < cnt) shared_pair<MODE>(w, a, S, e, jbase + o, so, ro, mo, co, o0, okk);
    }
    __syncwarp();
    if (mine) {
      for (uint32_t i = r0; i < r0 + kk; ++i) {
        const uint32_t f = S.fl[i];
        if (!(f & 1u)) continue;
        if (f & 2u) p = add(p, (f & 4u) ? v2(0.01f, 0.0f) : v2(-0.01f, -0.0f));
        p = add(p, v2(S.cx[i], S.cy[i]));
        if (f & 4u) {
          ++ncontacts;
          npush += (f >> 1) & 1u;
        }
      }
    }
    __syncwarp();
    base = end;
  }
  return p;
}

// Storage slot i -> its position in this substep's cell order.
__global__ void __launch_bounds__(256) k_permute(WorldDev w, SingleArgs a) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n_bodies) return;
  const uint32_t key = w.key[i];
  const uint32_t j = w.cell_start[key] + w.rank[i];
  if (j >= w.n_bodies) {
    atomicOr(w.status, ST_BAD_INDEX);
    return;
  }
  const float4 av = a.a_in[i];
  a.a_out[j] = av;
  a.b_out[j] = a.b_in[i];
  if (a.move_v) a.v_out[j] = a.v_in[i];
  w.ckey[j] = key;
  const uint32_t id = __float_as_uint(av.w);
  if (id < w.n_bodies) w.where[id] = j;
}

// Cell-order copy of the snapshot records (candidates of this substep).
__global__ void __launch_bounds__(256) k_scatter_cand(WorldDev w, const float4* __restrict__ a_in,
                                                      float4* __restrict__ cand) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n_bodies) return;
  const uint32_t j = w.cell_start[w.key[i]] + w.rank[i];
  if (j >= w.n_bodies) {
    atomicOr(w.status, ST_BAD_INDEX);
    return;
  }
  cand[j] = a_in[i];
}

// HOOKS: compiled with the adjoint's contact recording and the collision
// event stream.  A body whose 3x3 cells hold too many candidates for its
// near mask, or which has more near candidates than its phase 2 takes
// (WARP_NEAR shared over the warp, DEFER_NEAR per lane), is left to
// k_step_deferred: one such body would hold its whole warp in the
// O(contacts x candidates) walk or the O(near^2) ordered selection.
template <int MODE, bool HOOKS>
__global__ void __launch_bounds__(STEP_THREADS, 8) k_step_single(WorldDev w, SingleArgs a) {
  // phase 2 shared out over the warp (apply_near_warp): the plain step of a
  // uniform world
  constexpr bool WARP2 = MODE == 0 && !HOOKS;
  // phase 2 of the others: near candidate ids and positions,
  // thread-interleaved
  __shared__ uint32_t s_ids[WARP2 ? 1 : DEFER_NEAR * STEP_THREADS], s_qs[WARP2 ? 1 : DEFER_NEAR * STEP_THREADS];
  // event stream: the partners of this thread's events of phase 2, appended
  // together by the warp after it
  __shared__ uint32_t s_ev[HOOKS ? DEFER_NEAR * STEP_THREADS : 1];
  // the near pairs of each warp
  __shared__ PairSlots s_pairs[WARP2 ? STEP_THREADS / 32 : 1];
  uint32_t nev = 0;
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  const bool live = j < w.n_bodies;
  uint32_t ncontacts = 0, npush = 0;
  bool deferred = false;  // contacts (and the rest of the body's substep) left to k_step_deferred
  // this lane's near candidates for the warp's phase 2
  unsigned long long wnear = 0ull;
  uint32_t ws0 = 0, ws1 = 0, ws2 = 0, wt1 = 0, wt2 = 0;
  float4 av = make_float4(0.0f, 0.0f, 0.0f, 0.0f), bv = av;
  uint32_t c = 0;
  const WorldParam wp0 = w.wparam[0];
  BodyConst k;
  k.m = 0.0f;
  float2 p0 = v2(0.0f, 0.0f), p = p0;
  uint32_t nrec = 0;  // contacts recorded for the adjoint
  if (live) {
    av = a.a_in[j];
    bv = a.b_in[j];
    c = __float_as_uint(av.w);
    if (c >= w.n_bodies) {
      atomicOr(w.status, ST_BAD_INDEX);
      c = 0;
    }
    const float2 s = v2(av.x, av.y);
    const float r = av.z;
    k = body_const<MODE>(w, wp0, c, r);
    const WorldParam wp = MODE == 2 ? w.wparam[k.world] : wp0;
    p0 = v2(bv.x, bv.y);  // position at the start of the substep
    p = p0;

    const uint32_t own_key = a.contacts ? a.own_cell[j] : 0u;
    const uint32_t wm = (1u << wp.log2w) - 1u, hm = (1u << wp.log2h) - 1u;
    const uint32_t lx = (own_key - wp.cell_base) & wm, ly = (own_key - wp.cell_base) >> wp.log2w;
    const bool interior = lx >= 1u && lx < wm && ly >= 1u && ly < hm;
    if (a.contacts && interior) {
      // Cells away from the grid edge: the 3x3 block is three contiguous
      // ranges of the cell-order array, one per row.
      const float4* __restrict__ C = a.cand;
      const uint32_t n = w.n_bodies;
      const uint32_t r1 = own_key - 1u, r0 = r1 - (wm + 1u), r2 = r1 + (wm + 1u);
      const uint32_t s0 = w.cell_start[r0], s1 = w.cell_start[r1], s2 = w.cell_start[r2];
      const uint32_t e0 = min(w.cell_start[r0 + 3u], n), e1 = min(w.cell_start[r1 + 3u], n),
                     e2 = min(w.cell_start[r2 + 3u], n);
      const uint32_t l0 = e0 > s0 ? e0 - s0 : 0u, l1 = e1 > s1 ? e1 - s1 : 0u, l2 = e2 > s2 ? e2 - s2 : 0u;
      // bit positions are padded to multiples of 4 per row: they must fit 64
      if (((l0 + 3u) & ~3u) + ((l1 + 3u) & ~3u) + ((l2 + 3u) & ~3u) <= 64u) {
        // Phase 1: squared-distance test per candidate (self excluded); near
        // candidates become bits of their position (row 0 at bit 0, row 1
        // at bit 4*ceil(l0/4), ...).
        unsigned long long nb = 0ull;
        uint32_t t = 0;
        near_range(C, s, r, c, s0, s0 + l0, t, nb);
        const uint32_t t1 = t;
        near_range(C, s, r, c, s1, s1 + l1, t, nb);
        const uint32_t t2 = t;
        near_range(C, s, r, c, s2, s2 + l2, t, nb);
        // Phase 2: the near candidates in ascending arena id
        if ((uint32_t)__popcll(nb) > (WARP2 ? WARP_NEAR : DEFER_NEAR)) {
          deferred = true;
        } else if (!WARP2) {
          p = apply_near_s<MODE, HOOKS>(w, a, nb, s0, s1, s2, t1, t2, j, c, p0, s, r, k.m, ncontacts, npush, nrec,
                                        s_ids + threadIdx.x, s_qs + threadIdx.x,
                                        s_ev + (HOOKS ? threadIdx.x : 0u), nev);
        } else {
          wnear = nb;
          ws0 = s0;
          ws1 = s1;
          ws2 = s2;
          wt1 = t1;
          wt2 = t2;
        }
      } else {
        deferred = true;
      }
    } else if (a.contacts) {
      // cells on the grid edge (the torus wraps): general segments
      const float4* __restrict__ C = a.cand;
      const Segments g = segments(w, wp, own_key);
      const uint32_t total = g.l[0] + g.l[1] + g.l[2] + g.l[3] + g.l[4] + g.l[5];
      if (total <= 64u) {
        // Phase 1: one squared-distance test per candidate (self included:
        // it is skipped below); near candidates become bits of their
        // position in the 3x3 enumeration.
        unsigned long long nb = 0ull;
        uint32_t t = 0;
#pragma unroll
        for (int sg = 0; sg < 6; ++sg) {
          const uint32_t q1 = g.s[sg] + g.l[sg];
          for (uint32_t q = g.s[sg]; q < q1; ++q, ++t) {
            const float4 o = C[q];
            if (near_pair(s.x - o.x, s.y - o.y, r + o.z)) nb |= 1ull << t;
          }
        }
        // Phase 2: the near candidates in ascending arena id (the
        // reference's pair order for this body), the warp's lanes in step.
        while (nb) {
          unsigned long long best_bit = 0ull;
          uint32_t best = 0xffffffffu;
          float4 bo = make_float4(0.f, 0.f, 0.f, 0.f);
          for (unsigned long long mk = nb; mk; mk &= mk - 1ull) {
            const float4 o = C[slot_of(g, (uint32_t)(__ffsll((long long)mk) - 1))];
            const uint32_t c2 = __float_as_uint(o.w);
            if (c2 < best) {
              best = c2;
              bo = o;
              best_bit = mk & (~mk + 1ull);
            }
          }
          nb &= ~best_bit;
          if (best >= w.n_bodies || best == c) continue;
          const float m2 = (MODE == 0 || a.mass4r) ? bo.z * 4.0f : w.body_c[best].x;
          SinglePair sp;
          if (!single_pair(w, a, c, p0, s, r, k.m, best, v2(bo.x, bo.y), bo.z, m2, sp)) continue;
          if (sp.pushed) p = add(p, sp.push);
          p = add(p, sp.corr);
          if (HOOKS && a.rec_list) record_contact(w, a, c, best, sp.pushed, nrec);
          if (best < c) {
            ++ncontacts;
            npush += sp.pushed ? 1u : 0u;
            if (HOOKS && w.ev_rec) single_event(w, a, c, j, best);
          }
        }
      } else {
        deferred = true;
      }
    }
    if (!WARP2 && !deferred) {
      if (HOOKS && a.rec_list) {
        a.rec_n[c] = nrec;
        if (nrec) atomicMax(a.rec_max, nrec);
      }
      finish_single<MODE>(w, a, wp, k, j, c, av, bv, p0, p);
    }
  }
  if (WARP2) {
    // (a warp without near candidates skips phase 2)
    if (a.contacts && __any_sync(0xffffffffu, wnear != 0ull))
      p = apply_near_warp<MODE>(w, a, s_pairs[threadIdx.x >> 5], lane, j - lane, wnear, ws0, ws1, ws2, wt1, wt2, c,
                                v2(av.x, av.y), av.z, k.m, p, ncontacts, npush);
    // the records again (cache hits) rather than registers held across
    // phase 2
    if (live && !deferred) finish_single<MODE>(w, a, wp0, k, j, c, a.a_in[j], a.b_in[j], p0, p);
  }
  if (HOOKS && w.ev_rec) {
    // phase 2's events of the warp: one atomic for all of them
    uint32_t incl = nev;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (total) {
      if (lane == 0) base = atomicAdd(w.ev_count, total);
      base = __shfl_sync(0xffffffffu, base, 0);
    }
    if (nev) {
      const uint32_t seq = *w.ev_seq;
      const uint32_t c = __float_as_uint(a.a_in[j].w);
      const float2 va = a.v_in[j];
      // four events at a time: their partners' slot and velocity loads in
      // flight together
      for (uint32_t i0 = 0; i0 < nev; i0 += 4u) {
        uint32_t lo[4], jl[4];
        float2 vb[4];
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u) lo[u] = i0 + u < nev ? s_ev[(i0 + u) * STEP_THREADS + threadIdx.x] : 0u;
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u) jl[u] = i0 + u < nev ? w.where[lo[u]] : 0u;
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u) vb[u] = i0 + u < nev && jl[u] < w.n_bodies ? a.v_in[jl[u]] : v2(0.0f, 0.0f);
#pragma unroll
        for (uint32_t u = 0; u < 4u; ++u) {
          if (i0 + u >= nev) break;
          const uint32_t slot = base + (incl - nev) + i0 + u;
          if (jl[u] >= w.n_bodies) {
            atomicOr(w.status, ST_BAD_INDEX);
            continue;
          }
          if (slot < w.ev_cap) {
            w.ev_rec[slot] = make_uint4(seq, c, lo[u], 0u);
            w.ev_vel[slot] = make_float4(va.x, va.y, vb[u].x, vb[u].y);
          }
        }
      }
    }
  }
  if (a.contacts) {
    // append the deferred bodies to the list k_step_deferred works through
    const uint32_t dm = __ballot_sync(0xffffffffu, deferred);
    if (dm) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(w.defer_count, (uint32_t)__popc(dm));
      base = __shfl_sync(0xffffffffu, base, 0);
      const uint32_t at = base + (uint32_t)__popc(dm & ((1u << lane) - 1u));
      if (deferred) {
        if (at < w.n_bodies) w.defer_list[at] = j;
        else atomicOr(w.status, ST_BAD_INDEX);
      }
    }
  }
  if (a.contacts) count_warp(w, ncontacts, npush, deferred);
}

// The bodies k_step_single deferred (many candidates or many near
// candidates), one warp each: the warp's lanes test the 3x3 candidates
// together with the reference's exact test and compute each contact's
// correction (each depends only on the snapshots, masses and start-of-substep
// positions), the contacts are ranked by partner id in shared memory, and
// one lane applies them in that order -- the reference's pair order for this
// body -- then finishes the body's substep.  More than DEFER_CAP contacts:
// the exact selection walk on one lane.
template <int MODE, bool HOOKS>
__global__ void __launch_bounds__(DEFER_THREADS) k_step_deferred(WorldDev w, SingleArgs a) {
  __shared__ DeferWarp dsm[DEFER_THREADS / 32];
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  DeferWarp& S = dsm[wib];
  const uint32_t n = w.n_bodies;
  const uint32_t n_def = min(*w.defer_count, n);
  const uint32_t gw = blockIdx.x * (DEFER_THREADS / 32) + wib, nwarps = gridDim.x * (DEFER_THREADS / 32);
  const WorldParam wp0 = w.wparam[0];
  uint32_t tc = 0, tp = 0;
  for (uint32_t it = gw; it < n_def; it += nwarps) {
    const uint32_t j = w.defer_list[it];
    if (j >= n) {
      if (lane == 0) atomicOr(w.status, ST_BAD_INDEX);
      continue;
    }
    const float4 av = a.a_in[j], bv = a.b_in[j];
    uint32_t c = __float_as_uint(av.w);
    if (c >= n) {
      if (lane == 0) atomicOr(w.status, ST_BAD_INDEX);
      c = 0;
    }
    const float2 s = v2(av.x, av.y);
    const float r = av.z;
    const BodyConst k = body_const<MODE>(w, wp0, c, r);
    const WorldParam wp = MODE == 2 ? w.wparam[k.world] : wp0;
    const float2 p0 = v2(bv.x, bv.y);
    const Segments g = segments(w, wp, a.own_cell[j]);
    const uint32_t m = g.l[0] + g.l[1] + g.l[2] + g.l[3] + g.l[4] + g.l[5];
    uint32_t cnt = 0;
    for (uint32_t t0 = 0; t0 < m; t0 += 32u) {
      const uint32_t t = t0 + lane;
      bool hit = false;
      SinglePair sp;
      uint32_t c2 = 0;
      if (t < m) {
        const float4 o = a.cand[slot_of(g, t)];
        c2 = __float_as_uint(o.w);
        if (c2 != c && c2 < n) {
          const float m2 = (MODE == 0 || a.mass4r) ? o.z * 4.0f : w.body_c[c2].x;
          hit = single_pair(w, a, c, p0, s, r, k.m, c2, v2(o.x, o.y), o.z, m2, sp);
        }
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, hit);
      const uint32_t at = cnt + (uint32_t)__popc(bal & ((1u << lane) - 1u));
      if (hit && at < DEFER_CAP) {
        S.id[at] = c2;
        S.corr[at] = make_float4(sp.corr.x, sp.corr.y, __uint_as_float(sp.pushed ? 1u : 0u), 0.0f);
      }
      cnt += (uint32_t)__popc(bal);
    }
    __syncwarp();
    if (cnt <= DEFER_CAP) {
      // rank of every contact by partner id (ids are distinct)
      for (uint32_t e = lane; e < cnt; e += 32u) {
        const uint32_t ide = S.id[e];
        uint32_t rank = 0;
        for (uint32_t f = 0; f < cnt; ++f) rank += S.id[f] < ide ? 1u : 0u;
        S.order[rank] = e;
      }
      __syncwarp();
      if (HOOKS && w.ev_rec) {
        // the body's events (its contacts with lower ids), appended by all
        // lanes; the host puts the buffer in the reference's order
        const uint32_t seq = *w.ev_seq;
        const float2 va = a.v_in[j];
        for (uint32_t e0 = 0; e0 < cnt; e0 += 32u) {
          const uint32_t e = e0 + lane;
          const uint32_t c2 = e < cnt ? S.id[e] : 0xffffffffu;
          const bool ev = c2 < c;
          const uint32_t jl = ev ? w.where[c2] : 0u;
          const uint32_t bal = __ballot_sync(0xffffffffu, ev);
          uint32_t base = 0;
          if (lane == 0 && bal) base = atomicAdd(w.ev_count, (uint32_t)__popc(bal));
          base = __shfl_sync(0xffffffffu, base, 0);
          const uint32_t slot = base + (uint32_t)__popc(bal & ((1u << lane) - 1u));
          if (ev && jl >= n) atomicOr(w.status, ST_BAD_INDEX);
          if (ev && slot < w.ev_cap) {
            const float2 vb = jl < n ? a.v_in[jl] : v2(0.0f, 0.0f);
            w.ev_rec[slot] = make_uint4(seq, c, c2, 0u);
            w.ev_vel[slot] = make_float4(va.x, va.y, vb.x, vb.y);
          }
        }
      }
      if (lane == 0) {
        float2 p = p0;
        uint32_t nrec = 0;
        for (uint32_t i = 0; i < cnt; ++i) {
          const uint32_t e = S.order[i];
          if (e >= cnt) {  // ranks are a permutation when the partner ids are distinct
            atomicOr(w.status, ST_BAD_INDEX);
            continue;
          }
          const uint32_t c2 = S.id[e];
          const float4 cr = S.corr[e];
          const bool pushed = __float_as_uint(cr.z) != 0u;
          if (pushed) p = add(p, c > c2 ? v2(0.01f, 0.0f) : v2(-0.01f, -0.0f));
          p = add(p, v2(cr.x, cr.y));
          if (HOOKS && a.rec_list) record_contact(w, a, c, c2, pushed, nrec);
          if (c2 < c) {
            ++tc;
            tp += pushed ? 1u : 0u;
          }
        }
        if (HOOKS && a.rec_list) {
          a.rec_n[c] = nrec;
          if (nrec) atomicMax(a.rec_max, nrec);
        }
        finish_single<MODE>(w, a, wp, k, j, c, av, bv, p0, p);
      }
    } else if (lane == 0) {
      uint32_t nc = 0, np = 0, nr = 0;
      const float2 p = contacts_walk<MODE, HOOKS>(w, a, g, j, c, p0, s, r, k.m, nc, np, nr);
      tc += nc;
      tp += np;
      if (HOOKS && a.rec_list) {
        a.rec_n[c] = nr;
        if (nr) atomicMax(a.rec_max, nr);
      }
      finish_single<MODE>(w, a, wp, k, j, c, av, bv, p0, p);
    }
    __syncwarp();
  }
  if (lane == 0 && (tc || tp)) {
    const uint32_t bin = gw & (COUNTER_BINS - 1);
    if (tc) {
      atomicAdd(w.contacts_total + bin, (unsigned long long)tc);
      atomicAdd(w.contacts_sub + bin, tc);
    }
    if (tp) atomicAdd(w.pushouts_total + bin, (unsigned long long)tp);
  }
}

// Keys and ranks of the current storage (after a load or a host write).
__global__ void __launch_bounds__(256) k_keys_single(WorldDev w, const float4* __restrict__ A, int mode) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= w.n_bodies) return;
  const float4 a = A[j];
  const uint32_t c = __float_as_uint(a.w);
  const uint32_t world = mode == 2 ? rec_world(w.body_c[c < w.n_bodies ? c : 0u]) : 0u;
  const uint32_t key = cell_key(w.wparam[world], v2(a.x, a.y));
  w.key[j] = key;
  w.rank[j] = atomicAdd(w.cell_count + key, 1u);
}

// Storage order -> arena order (reads) and back (host writes).
__global__ void __launch_bounds__(256) k_gather_single(WorldDev w, const float4* __restrict__ A,
                                                       const float4* __restrict__ B, const float2* __restrict__ V,
                                                       float2* pos, float2* pos_old, float2* vel, float2* snap,
                                                       float v_div) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= w.n_bodies) return;
  const float4 a = A[j];
  const uint32_t c = __float_as_uint(a.w);
  if (c >= w.n_bodies) {
    atomicOr(w.status, ST_BAD_INDEX);
    return;
  }
  const float4 b = B[j];
  if (pos) pos[c] = v2(b.x, b.y);
  if (pos_old) pos_old[c] = v2(b.z, b.w);
  if (vel) {
    // V holds the last substep's displacement when v_div != 0 (static
    // bodies store 0, and 0 / dt = 0)
    const float2 v = V[j];
    vel[c] = v_div != 0.0f ? divs(v, v_div) : v;
  }
  if (snap) snap[c] = v2(a.x, a.y);
}

__global__ void __launch_bounds__(256) k_write_single(WorldDev w, float4* A, float4* B, float2* V,
                                                      const float2* pos, const float2* pos_old, const float2* vel,
                                                      const float2* snap) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= w.n_bodies) return;
  const uint32_t c = __float_as_uint(A[j].w);
  if (c >= w.n_bodies) {
    atomicOr(w.status, ST_BAD_INDEX);
    return;
  }
  float4 b = B[j];
  if (pos) {
    const float2 p = pos[c];
    b.x = p.x;
    b.y = p.y;
  }
  if (pos_old) {
    const float2 p = pos_old[c];
    b.z = p.x;
    b.w = p.y;
  }
  B[j] = b;
  if (vel) V[j] = vel[c];
  if (snap) {
    const float2 q = snap[c];
    A[j].x = q.x;
    A[j].y = q.y;
  }
}

// ---------------------------------------------------------------------------
static inline uint32_t nblocks(uint32_t n) { return (n + 255u) / 256u; }

void launch_permute(const WorldDev& w, const SingleArgs& a, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_permute<<<nblocks(w.n_bodies), 256, 0, st>>>(w, a);
}

void launch_scatter_cand(const WorldDev& w, const float4* a_in, float4* cand, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_scatter_cand<<<nblocks(w.n_bodies), 256, 0, st>>>(w, a_in, cand);
}

void launch_step_single(const WorldDev& w, const SingleArgs& a, int mode, cudaStream_t st) {
  if (!w.n_bodies) return;
  const uint32_t g = (w.n_bodies + STEP_THREADS - 1) / STEP_THREADS;
  if (a.rec_list || w.ev_rec) {
    if (mode == 0) k_step_single<0, true><<<g, STEP_THREADS, 0, st>>>(w, a);
    else if (mode == 1) k_step_single<1, true><<<g, STEP_THREADS, 0, st>>>(w, a);
    else k_step_single<2, true><<<g, STEP_THREADS, 0, st>>>(w, a);
  } else {
    if (mode == 0) k_step_single<0, false><<<g, STEP_THREADS, 0, st>>>(w, a);
    else if (mode == 1) k_step_single<1, false><<<g, STEP_THREADS, 0, st>>>(w, a);
    else k_step_single<2, false><<<g, STEP_THREADS, 0, st>>>(w, a);
  }
}

void launch_step_deferred(const WorldDev& w, const SingleArgs& a, int mode, cudaStream_t st) {
  if (!w.n_bodies || !w.defer_list) return;
  if (a.rec_list || w.ev_rec) {
    if (mode == 0) k_step_deferred<0, true><<<DEFER_BLOCKS, DEFER_THREADS, 0, st>>>(w, a);
    else if (mode == 1) k_step_deferred<1, true><<<DEFER_BLOCKS, DEFER_THREADS, 0, st>>>(w, a);
    else k_step_deferred<2, true><<<DEFER_BLOCKS, DEFER_THREADS, 0, st>>>(w, a);
  } else {
    if (mode == 0) k_step_deferred<0, false><<<DEFER_BLOCKS, DEFER_THREADS, 0, st>>>(w, a);
    else if (mode == 1) k_step_deferred<1, false><<<DEFER_BLOCKS, DEFER_THREADS, 0, st>>>(w, a);
    else k_step_deferred<2, false><<<DEFER_BLOCKS, DEFER_THREADS, 0, st>>>(w, a);
  }
}

void launch_keys_single(const WorldDev& w, const float4* A, int mode, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_keys_single<<<nblocks(w.n_bodies), 256, 0, st>>>(w, A, mode);
}

void launch_gather_single(const WorldDev& w, const float4* A, const float4* B, const float2* V, float2* pos,
                          float2* pos_old, float2* vel, float2* snap, float v_div, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_gather_single<<<nblocks(w.n_bodies), 256, 0, st>>>(w, A, B, V, pos, pos_old, vel, snap, v_div);
}

void launch_write_single(const WorldDev& w, float4* A, float4* B, float2* V, const float2* pos,
                         const float2* pos_old, const float2* vel, const float2* snap, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_write_single<<<nblocks(w.n_bodies), 256, 0, st>>>(w, A, B, V, pos, pos_old, vel, snap);
}

}  // namespace blobs
