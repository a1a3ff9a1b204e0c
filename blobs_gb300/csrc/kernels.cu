// kernels.cu -- sm_103a kernels of one blobs substep (physics.rs:397-422)
// on the general path (several colliders per body, offsets, groups, sensors,
// joints), and the cell scan both paths share.  The single-sphere path's
// kernels are in single.cu.
//
// Per substep, for every packed world at once:
//   k_tile_sums,       exclusive scan of the per-cell collider counts -> cell
//   k_scan_apply       ranges (two wait-free kernels), counts reset
//   k_scatter_forces   counting-sort scatter of the colliders into cell order
//                      (the one-digit LSD radix pass over the cell key) and,
//                      when springs exist, gravity + spring forces per body
//   k_collider_contacts  per cell-sorted collider: its contacts over the 3x3
//                      cells (pair key, correction of its body)
//   k_body_contacts    per body: its colliders' contacts applied in the
//                      reference's pair-sequence order; fused with
//                      integration when there are no joints
//   k_contact_single   both passes in one for single-collider bodies
//   k_joint_blocks     the small joint components, each swept alone in the
//                      reference's order in shared memory
//   k_joints           one colour of the large components' joints
//   k_integrate        Verlet + collider snapshot + constraints, and the cell
//                      key / rank of every collider for the next substep
//
// The cell counts for substep s+1 are produced by the integration of substep
// s (atomicAdd rank per collider), so no separate key pass runs in steady
// state.  Compiled with --fmad=false; see device.cuh.
#include "device.cuh"
#include "kernels.h"

namespace blobs {

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void set_status(const WorldDev& w, uint32_t bit) { atomicOr(w.status, bit); }

__device__ __forceinline__ WorldParam load_wparam(const WorldDev& w, uint32_t world) {
  return w.wparam[world];
}


// ---------------------------------------------------------------------------
// Cell scan in two wait-free kernels: k_tile_sums reduces each tile of
// SCAN_TILE cell counts; k_scan_apply gives every tile its prefix by summing
// the sums of all earlier tiles (with more than SCAN_PREFIX_TILES tiles,
// k_tile_prefix computes those prefixes once, in between), then writes
// cell_start[k] = sum(cell_count[0..k)), cell_start[n] = total, and resets
// cell_count to zero for the next substep.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_warp) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) s_warp[warp] = v;
  __syncthreads();
  uint32_t t = 0;
  if (warp == 0) {
    t = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;  // valid in warp 0
}

__device__ __forceinline__ void load_tile(const WorldDev& w, size_t base, uint32_t* v, bool zero) {
  const uint32_t n = w.n_cells;
  if (base + SCAN_ITEMS <= n) {
    uint4* src = reinterpret_cast<uint4*>(w.cell_count + base);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
      const uint4 t = src[q];
      v[4 * q + 0] = t.x;
      v[4 * q + 1] = t.y;
      v[4 * q + 2] = t.z;
      v[4 * q + 3] = t.w;
      if (zero) src[q] = make_uint4(0u, 0u, 0u, 0u);
    }
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const size_t k = base + i;
      v[i] = k < n ? w.cell_count[k] : 0u;
      if (zero && k < n) w.cell_count[k] = 0u;
    }
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_tile_sums(WorldDev w) {
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  load_tile(w, base, v, false);
  uint32_t t = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) t += v[i];
  t = block_sum(t, s_warp);
  if (threadIdx.x == 0) w.tile_sums[blockIdx.x] = t;
  if (blockIdx.x == 0 && threadIdx.x < COUNTER_BINS) {
    if (w.contacts_sub) w.contacts_sub[threadIdx.x] = 0u;
    if (w.defer_sub) w.defer_sub[threadIdx.x] = 0u;
    if (threadIdx.x == 0 && w.defer_count) *w.defer_count = 0u;
  }
}

// Many tiles (large or batched grids): one block turns the tile sums into
// their exclusive prefix in place, so that k_scan_apply reads its prefix
// instead of summing all earlier tiles (quadratic in the tile count).
__global__ void __launch_bounds__(1024) k_tile_prefix(WorldDev w) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_carry;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0u;
  __syncthreads();
  for (uint32_t base = 0; base < w.n_tiles; base += 1024u) {
    const uint32_t t = base + threadIdx.x;
    const uint32_t v = t < w.n_tiles ? w.tile_sums[t] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t u = s_warp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
        if (lane >= (uint32_t)o) u += y;
      }
      s_warp[lane] = u;
    }
    __syncthreads();
    const uint32_t carry = s_carry;
    if (t < w.n_tiles) w.tile_sums[t] = carry + (warp ? s_warp[warp - 1] : 0u) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = carry + s_warp[31];
    __syncthreads();
  }
}

template <bool PREFIXED>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(WorldDev w) {
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ uint32_t s_prefix;
  if (PREFIXED) {
    if (threadIdx.x == 0) s_prefix = w.tile_sums[blockIdx.x];
  } else {
    // prefix of this tile = sum of the sums of tiles [0, blockIdx.x)
    uint32_t p = 0;
    for (uint32_t t = threadIdx.x; t < blockIdx.x; t += SCAN_THREADS) p += w.tile_sums[t];
    p = block_sum(p, s_warp);
    if (threadIdx.x == 0) s_prefix = p;
  }
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  load_tile(w, base, v, true);
  uint32_t tsum = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) tsum += v[i];
  // exclusive scan of the thread sums across the block
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = tsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  __syncthreads();  // s_warp reuse
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    constexpr int NW = SCAN_THREADS / 32;
    uint32_t t = lane < NW ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < NW; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (uint32_t)o) t += y;
    }
    if (lane < NW) s_warp[lane] = t;
  }
  __syncthreads();
  uint32_t run = s_prefix + (warp ? s_warp[warp - 1] : 0u) + x - tsum;
  const uint32_t n = w.n_cells;
  if (base + SCAN_ITEMS <= n) {
    uint4* dst = reinterpret_cast<uint4*>(w.cell_start + base);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
      uint4 t;
      t.x = run; run += v[4 * q + 0];
      t.y = run; run += v[4 * q + 1];
      t.z = run; run += v[4 * q + 2];
      t.w = run; run += v[4 * q + 3];
      dst[q] = t;
    }
    if (base + SCAN_ITEMS == n) w.cell_start[n] = run;
  } else {
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const size_t k = base + i;
      if (k < n) {
        w.cell_start[k] = run;
        run += v[i];
        if (k + 1 == n) w.cell_start[n] = run;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// gravity + springs for one body (physics.rs:369-375, springs.rs:25-47,
// rigid_body.rs:155-160).  Springs are visited in ascending arena index and
// each spring force is recomputed with identical operations at both
// endpoints, so every body accumulates exactly the reference's sequence.
// ---------------------------------------------------------------------------
template <bool PEND>
__device__ __forceinline__ float2 body_forces(const WorldDev& w, uint32_t b, const float2* __restrict__ pos) {
  float2 a = PEND ? w.pend_acc[b] : v2(0.0f, 0.0f);
  a = add(a, mul(w.gravity, w.gmod[b]));
  const float m = w.mass[b];
  const uint32_t q0 = w.body_spr_start[b], q1 = w.body_spr_start[b + 1];
  for (uint32_t q = q0; q < q1; ++q) {
    const uint32_t e = w.body_spr[q];
    const uint32_t s = e >> 1;
    const uint32_t ia = w.spr_a[s], ib = w.spr_b[s];
    const float2 pa = pos[ia], pb = pos[ib];
    const float2 d = sub(pb, pa);
    const float dist = len2(d);
    const float2 dir = divs(d, dist);
    const float2 rv = sub(w.vel[ia], w.vel[ib]);
    const float2 damping = mul(dir, w.spr_c[s] * dot2(rv, dir));
    const float sk = w.spr_k[s] * (dist - w.spr_rest[s]);
    const float2 fm = v2(sk - damping.x, sk - damping.y);  // f32 - Vec2 broadcast, springs.rs:41
    float2 f = mulv(dir, fm);
    if (e & 1u) f = v2(-f.x, -f.y);
    a = add(a, divs(f, m));
  }
  return a;
}

template <bool MW, bool SCATTER, bool SPR, bool PEND>
__global__ void __launch_bounds__(256) k_scatter_forces(WorldDev w, const float2* __restrict__ pos) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (SCATTER) {
    if (i < w.n_cols) {
      const float2 s = w.snap[i];
      const WorldParam wp = load_wparam(w, MW ? w.col_world[i] : 0u);
      const uint32_t key = cell_key(wp, s);
      const uint32_t slot = w.cell_start[key] + w.rank[i];
      if (slot < w.n_cols) w.sorted[slot] = make_float4(s.x, s.y, w.col_radius[i], __uint_as_float(i));
      else set_status(w, ST_BAD_INDEX);
    }
  }
  if (SPR && i < w.n_bodies) {
    if (!(w.bflags[i] & BF_STATIC)) w.acc[i] = body_forces<PEND>(w, i, pos);
  }
}

// ---------------------------------------------------------------------------
// integration of one body (physics.rs:323-367) followed by the constraints
// (physics.rs:377-395, then the wall extension).  `p` is the body position
// after contacts and joints.  Collider snapshots are taken BEFORE the
// constraints (the reference refreshes them inside update_objects only), and
// their cell keys/ranks for the next substep are recorded here.
// ---------------------------------------------------------------------------
template <bool MW, bool SPR, bool PEND, bool SINGLE>
__device__ __forceinline__ void integrate_body(const WorldDev& w, uint32_t b, float2 p, float2* __restrict__ pos_out,
                                               const SubstepArgs& a) {
  const uint8_t fl = w.bflags[b];
  const float dt = a.dt;
  float2 po;
  float2 vel;
  float rot = 0.0f;
  if (!SINGLE || a.rot_dynamic) rot = w.rot[b];
  if (fl & BF_STATIC) {
    po = p;
    vel = v2(0.0f, 0.0f);
  } else {
    po = w.pos_old[b];
    if (PEND && (fl & BF_VREQ)) po = sub(p, mul(w.vreq[b], dt));
    const float ratio = (fl & BF_FIRST_DYN) ? dt / a.old_dt : dt / dt;
    const float2 disp = mul(sub(p, po), ratio);
    float2 acc;
    if (SPR) {
      acc = w.acc[b];
    } else {
      acc = PEND ? w.pend_acc[b] : v2(0.0f, 0.0f);
      acc = add(acc, mul(w.gravity, w.gmod[b]));
    }
    po = p;
    p = add(p, add(disp, mul(mul(acc, dt), dt)));
    if (a.rot_dynamic) {
      const float tq = PEND ? w.pend_torque[b] : 0.0f;
      float av = w.angvel[b];
      av = av + (tq / w.inertia[b]) * dt;
      rot = rot + av * dt;
      w.angvel[b] = av;
      w.rot[b] = rot;
    }
    vel = divs(disp, dt);
  }
  const uint32_t world = MW ? w.body_world[b] : 0u;
  const WorldParam wp = load_wparam(w, world);
  if (SINGLE) {
    const float2 s = v2(0.0f + p.x, 0.0f + p.y);  // rot(θ) * 0 + p
    w.snap[b] = s;
    if (a.do_keys) w.rank[b] = atomicAdd(w.cell_count + cell_key(wp, s), 1u);
  } else {
    const uint32_t c0 = w.body_col_start[b], c1 = w.body_col_start[b + 1];
    for (uint32_t q = c0; q < c1; ++q) {
      const uint32_t c = w.body_cols[q];
      const float2 s = collider_translation(rot, p, w.col_off[c]);
      w.snap[c] = s;
      if (a.do_keys) w.rank[c] = atomicAdd(w.cell_count + cell_key(wp, s), 1u);
    }
  }
  for (uint32_t k = 0; k < w.n_circles; ++k) {
    const float2 c = v2(w.circles[3 * k], w.circles[3 * k + 1]);
    const float radius = w.circles[3 * k + 2];
    const float2 to = sub(p, c);
    const float dist = len2(to);
    if (dist > radius) p = add(c, mul(divs(to, dist), radius));
  }
  if (wp.has_box) {
    const float br = w.bound_r[b];
    p.x = fminf(fmaxf(p.x, wp.box_lo_x + br), wp.box_hi_x - br);
    p.y = fminf(fmaxf(p.y, wp.box_lo_y + br), wp.box_hi_y - br);
  }
  pos_out[b] = p;
  w.pos_old[b] = po;
  w.vel[b] = vel;
}

// ---------------------------------------------------------------------------
// Candidate enumeration: the 3 rows of 3 cells around point s, each row a
// contiguous range of the cell-sorted array (split in two where the torus
// wraps).
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ void for_each_candidate(const WorldDev& w, const WorldParam& wp, float2 s, F&& f) {
  const uint32_t wm = (1u << wp.log2w) - 1u, hm = (1u << wp.log2h) - 1u;
  const uint32_t ix = (uint32_t)grid_coord(s.x, wp.ox, wp.inv_cs), iy = (uint32_t)grid_coord(s.y, wp.oy, wp.inv_cs);
  const uint32_t x0 = (ix - 1u) & wm, x2 = (ix + 1u) & wm;
#pragma unroll 1
  for (int oy = -1; oy <= 1; ++oy) {
    const uint32_t row = wp.cell_base + (((iy + (uint32_t)oy) & hm) << wp.log2w);
    // ranges are clamped to the slot count: a corrupt cell table cannot walk
    // past the sorted array
    if (x0 < x2) {
      const uint32_t e0 = w.cell_start[row + x0], e1 = min(w.cell_start[row + x2 + 1u], w.n_cols);
      for (uint32_t e = e0; e < e1; ++e) f(e);
    } else {
      uint32_t e0 = w.cell_start[row + x0], e1 = min(w.cell_start[row + wm + 1u], w.n_cols);
      for (uint32_t e = e0; e < e1; ++e) f(e);
      e0 = w.cell_start[row], e1 = min(w.cell_start[row + x2 + 1u], w.n_cols);
      for (uint32_t e = e0; e < e1; ++e) f(e);
    }
  }
}

// One contact of collider c (body b) with collider c2 (body b2), in the
// reference's terms: a = the higher collider index (outer loop), b = lower.
// Returns false if the pair is not in contact.  Sets *push when the
// coincident-centre branch (physics.rs:272-286) was taken; its increments are
// then applied as (push, corr) in that order.
struct PairOut {
  float2 push;
  float2 corr;
  bool pushed;
  bool has_corr;
};

__device__ __forceinline__ bool contact_pair(const WorldDev& w, const float2* __restrict__ pos_in, uint32_t c,
                                             uint32_t b, float2 s, float r, float m_b, uint32_t c2, uint32_t b2,
                                             float2 s2, float r2, float m_b2, bool sensor_any, float2 off_c,
                                             float2 off_c2, PairOut& out) {
  const bool hi = c > c2;
  float2 axis = hi ? sub(s, s2) : sub(s2, s);
  float d = len2(axis);
  const float min_dist = hi ? (r + r2) : (r2 + r);
  if (!(d < min_dist)) return false;
  out.pushed = false;
  out.push = v2(0.0f, 0.0f);
  if (d < 1e-6f) {
    // Push-out with the snapshots refreshed to body position + offset.  The
    // positions used are those at the start of the contact pass (exact when
    // neither body received an earlier correction in this substep).
    const float2 pa = add(pos_in[hi ? b : b2], v2(0.01f, 0.0f));
    const float2 pb = sub(pos_in[hi ? b2 : b], v2(0.01f, 0.0f));
    const float2 sa = add(pa, hi ? off_c : off_c2);
    const float2 sb = add(pb, hi ? off_c2 : off_c);
    axis = sub(sa, sb);
    d = len2(axis);
    out.pushed = true;
    out.push = hi ? v2(0.01f, 0.0f) : v2(-0.01f, -0.0f);  // p - (0.01, 0) == p + (-0.01, -0)
  }
  out.has_corr = !sensor_any;
  out.corr = v2(0.0f, 0.0f);
  if (!sensor_any) {
    const float2 n = divs(axis, d);
    if (n.x != n.x || n.y != n.y) set_status(w, ST_NAN);
    const float delta = min_dist - d;
    const float ma = hi ? m_b : m_b2, mb = hi ? m_b2 : m_b;
    const float ratio = 1.0f - ma / (ma + mb);
    if (hi) {
      out.corr = mul(n, ratio * delta);
    } else {
      const float2 t = mul(n, (1.0f - ratio) * delta);
      out.corr = v2(-t.x, -t.y);
    }
  }
  return true;
}

__device__ __forceinline__ void sort_contacts(Contact* l, int n) {
  for (int i = 1; i < n; ++i) {
    Contact t = l[i];
    int j = i - 1;
    while (j >= 0 && l[j].key > t.key) {
      l[j + 1] = l[j];
      --j;
    }
    l[j + 1] = t;
  }
}

__device__ __forceinline__ unsigned long long pair_key(uint32_t c, uint32_t c2) {
  const uint32_t hi = c > c2 ? c : c2, lo = c > c2 ? c2 : c;
  return ((unsigned long long)hi << 33) | ((unsigned long long)lo << 1);
}

// Block-level sum of the contact / push-out counts, then one atomic per
// block into one of COUNTER_BINS bins (spreads same-address atomics over L2
// slices; the host sums the bins).  Every thread of the block must call it.
__device__ __forceinline__ void count_contacts(const WorldDev& w, uint32_t ncontacts, uint32_t npush) {
  __shared__ uint32_t s_c, s_p;
  if (threadIdx.x == 0) {
    s_c = 0u;
    s_p = 0u;
  }
  __syncthreads();
  uint32_t t = ncontacts, p = npush;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_down_sync(0xffffffffu, t, o);
    p += __shfl_down_sync(0xffffffffu, p, o);
  }
  if ((threadIdx.x & 31u) == 0) {
    if (t) atomicAdd(&s_c, t);
    if (p) atomicAdd(&s_p, p);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t bin = blockIdx.x & (COUNTER_BINS - 1);
    if (s_c) {
      atomicAdd(w.contacts_total + bin, (unsigned long long)s_c);
      atomicAdd(w.contacts_sub + bin, s_c);
    }
    if (s_p) atomicAdd(w.pushouts_total + bin, (unsigned long long)s_p);
  }
}

// ---------------------------------------------------------------------------
// k_contact_single: worlds whose bodies each own exactly one collider with a
// zero offset, default groups and no sensor.  One thread per cell-sorted
// slot, so a warp works on neighbouring cells.  Contacts are collected,
// sorted by the neighbour's arena index (= the reference's pair sequence for
// this body) and applied in that order; more than CONTACT_LIST contacts or a
// push-out switch to an exact selection walk.
// ---------------------------------------------------------------------------
template <bool MW, bool SPR, bool PEND, bool FUSE>
__global__ void __launch_bounds__(256) k_contact_single(WorldDev w, const float2* __restrict__ pos_in,
                                                        float2* __restrict__ pos_out, SubstepArgs args) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t ncontacts = 0, npush = 0;
  if (e < w.n_cols) {
    const float4 me = w.sorted[e];
    uint32_t c = __float_as_uint(me.w);
    if (c >= w.n_cols) {
      set_status(w, ST_BAD_INDEX);
      c = 0;
    }
    const float2 s = v2(me.x, me.y);
    const float r = me.z;
    const WorldParam wp = load_wparam(w, MW ? w.col_world[c] : 0u);
    const float m_c = w.mass[c];
    Contact list[CONTACT_LIST];
    int nl = 0;
    bool slow = false;
    for_each_candidate(w, wp, s, [&](uint32_t q) {
      if (q == e) return;
      const float4 o = w.sorted[q];
      const uint32_t c2 = __float_as_uint(o.w);
      if (c2 >= w.n_cols) return;
      if (!near_pair(s.x - o.x, s.y - o.y, r + o.z)) return;  // the exact test is made in contact_pair
      PairOut po;
      if (!contact_pair(w, pos_in, c, c, s, r, m_c, c2, c2, v2(o.x, o.y), o.z, w.mass[c2], false,
                        v2(0.0f, 0.0f), v2(0.0f, 0.0f), po))
        return;
      if (c > c2) {
        ++ncontacts;
        npush += po.pushed ? 1u : 0u;
        if (w.ev_rec) record_event(w, c, c2, w.vel[c], w.vel[c2]);
      }
      if (po.pushed || nl >= CONTACT_LIST) {
        slow = true;
        return;
      }
      list[nl].key = pair_key(c, c2);
      list[nl].corr = po.corr;
      ++nl;
    });
    float2 p = pos_in[c];
    if (!slow) {
      sort_contacts(list, nl);
      for (int k = 0; k < nl; ++k) p = add(p, list[k].corr);
    } else {
      // exact selection walk in ascending pair key
      unsigned long long last = 0ull;
      bool first = true;
      while (true) {
        unsigned long long best = ~0ull;
        PairOut bo;
        for_each_candidate(w, wp, s, [&](uint32_t q) {
          if (q == e) return;
          const float4 o = w.sorted[q];
          const uint32_t c2 = __float_as_uint(o.w);
          if (c2 >= w.n_cols) return;
          const unsigned long long k = pair_key(c, c2);
          if ((!first && k <= last) || k >= best) return;
          PairOut po;
          if (!contact_pair(w, pos_in, c, c, s, r, m_c, c2, c2, v2(o.x, o.y), o.z, w.mass[c2], false,
                            v2(0.0f, 0.0f), v2(0.0f, 0.0f), po))
            return;
          best = k;
          bo = po;
        });
        if (best == ~0ull) break;
        if (bo.pushed) p = add(p, bo.push);
        p = add(p, bo.corr);
        last = best;
        first = false;
      }
    }
    if (FUSE) {
      integrate_body<MW, SPR, PEND, true>(w, c, p, pos_out, args);
    } else {
      pos_out[c] = p;
    }
  }
  count_contacts(w, ncontacts, npush);
}

// ---------------------------------------------------------------------------
// The general contact pass: any body / collider layout (several colliders
// per body, offsets, groups, sensors), in two kernels.
//
// k_collider_contacts: one thread per cell-sorted collider slot (a warp works
// on neighbouring cells and every thread on one collider), which finds the
// collider's contacts and keeps up to CL_CAP of them -- (pair key,
// correction of its body) -- in clist.  A push-out, or more contacts, marks
// the body for the ordered walk.  Counts and events are taken here.
//
// k_body_contacts: one thread per body, which merges its colliders' contacts
// in the reference's pair-sequence order (outer collider index, then inner)
// and applies them; a marked body gathers its contacts again
// (collect_contacts), or on a push-out or a long list walks them in that
// order (ordered_walk), which also handles the push-out branch.
// ---------------------------------------------------------------------------
template <bool MW>
__global__ void __launch_bounds__(256) k_collider_contacts(WorldDev w, const float2* __restrict__ pos_in) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t ncontacts = 0, npush = 0;
  if (e < w.n_cols) {
    const float4 me = w.sorted[e];
    uint32_t c = __float_as_uint(me.w);
    if (c >= w.n_cols) {
      set_status(w, ST_BAD_INDEX);
      c = 0;
    }
    const uint32_t b = w.col_parent[c];
    const WorldParam wp = load_wparam(w, MW ? w.col_world[c] : 0u);
    const float2 s = v2(me.x, me.y);  // the snapshot and radius of collider c
    const float r = me.z;
    const float m_b = w.mass[b];
    const uint32_t memb = w.col_memb[c], filt = w.col_filt[c];
    const bool sens = w.col_sensor[c] != 0;
    const float2 off = w.col_off[c];
    Contact* out = w.clist + (size_t)c * CL_CAP;
    uint32_t n = 0;
    bool slow = false;
    for_each_candidate(w, wp, s, [&](uint32_t q) {
      const float4 o = w.sorted[q];
      const uint32_t c2 = __float_as_uint(o.w);
      if (c2 == c || c2 >= w.n_cols) return;
      const float2 s2 = v2(o.x, o.y);
      // squared-distance pre-test; the exact test is made in contact_pair
      if (!near_pair(s.x - s2.x, s.y - s2.y, r + o.z)) return;
      const uint32_t b2 = w.col_parent[c2];
      if (b2 == b) return;
      const uint32_t memb2 = w.col_memb[c2], filt2 = w.col_filt[c2];
      if (!((memb & filt2) != 0u && (memb2 & filt) != 0u)) return;
      const bool sens_any = sens || (w.col_sensor[c2] != 0);
      PairOut po;
      if (!contact_pair(w, pos_in, c, b, s, r, m_b, c2, b2, s2, o.z, w.mass[b2], sens_any, off, w.col_off[c2], po))
        return;
      if (c > c2) {
        ++ncontacts;
        npush += po.pushed ? 1u : 0u;
        if (w.ev_rec) record_event(w, c, c2, w.vel[b], w.vel[b2]);
      }
      if (po.pushed || n >= CL_CAP) {
        slow = true;
        return;
      }
      out[n].key = pair_key(c, c2);
      out[n].corr = po.corr;
      ++n;
    });
    w.ccount[c] = (uint8_t)n;
    if (slow) w.bslow[b] = 1u;
  }
  count_contacts(w, ncontacts, npush);
}

// All contacts of body b's colliders into `list`, in candidate order.
// Returns false on a push-out or more than CONTACT_LIST contacts.
__device__ __noinline__ bool collect_contacts(const WorldDev& w, const WorldParam& wp,
                                              const float2* __restrict__ pos_in, uint32_t b, uint32_t c0,
                                              uint32_t c1, float m_b, Contact* list, int& nl) {
  bool ok = true;
  for (uint32_t qc = c0; qc < c1 && ok; ++qc) {
    const uint32_t c = w.body_cols[qc];
    const float2 s = w.snap[c];
    const float r = w.col_radius[c];
    const uint32_t memb = w.col_memb[c], filt = w.col_filt[c];
    const bool sens = w.col_sensor[c] != 0;
    const float2 off = w.col_off[c];
    for_each_candidate(w, wp, s, [&](uint32_t q) {
      if (!ok) return;
      const float4 o = w.sorted[q];
      const uint32_t c2 = __float_as_uint(o.w);
      if (c2 == c || c2 >= w.n_cols) return;
      const uint32_t b2 = w.col_parent[c2];
      if (b2 == b) return;
      const uint32_t memb2 = w.col_memb[c2], filt2 = w.col_filt[c2];
      if (!((memb & filt2) != 0u && (memb2 & filt) != 0u)) return;
      const bool sens_any = sens || (w.col_sensor[c2] != 0);
      PairOut po;
      if (!contact_pair(w, pos_in, c, b, s, r, m_b, c2, b2, v2(o.x, o.y), o.z, w.mass[b2], sens_any, off,
                        w.col_off[c2], po))
        return;
      if (po.pushed || nl >= CONTACT_LIST) {
        ok = false;
        return;
      }
      list[nl].key = pair_key(c, c2);
      list[nl].corr = po.corr;
      ++nl;
    });
  }
  return ok;
}

// Body b's contacts applied one by one in pair-sequence order: each round
// selects the smallest pair key above the last one over all its colliders'
// candidates.
__device__ __noinline__ float2 ordered_walk(const WorldDev& w, const WorldParam& wp, const float2* __restrict__ pos_in,
                                            uint32_t b, uint32_t c0, uint32_t c1, float m_b) {
  float2 p = pos_in[b];
  unsigned long long last = 0ull;
  bool first = true;
  while (true) {
    unsigned long long best = ~0ull;
    PairOut bo;
    for (uint32_t qc = c0; qc < c1; ++qc) {
      const uint32_t c = w.body_cols[qc];
      const float2 s = w.snap[c];
      const float r = w.col_radius[c];
      const uint32_t memb = w.col_memb[c], filt = w.col_filt[c];
      const bool sens = w.col_sensor[c] != 0;
      const float2 off = w.col_off[c];
      for_each_candidate(w, wp, s, [&](uint32_t q) {
        const float4 o = w.sorted[q];
        const uint32_t c2 = __float_as_uint(o.w);
        if (c2 == c || c2 >= w.n_cols) return;
        const unsigned long long k = pair_key(c, c2);
        if ((!first && k <= last) || k >= best) return;
        const uint32_t b2 = w.col_parent[c2];
        if (b2 == b) return;
        const uint32_t memb2 = w.col_memb[c2], filt2 = w.col_filt[c2];
        if (!((memb & filt2) != 0u && (memb2 & filt) != 0u)) return;
        const bool sens_any = sens || (w.col_sensor[c2] != 0);
        PairOut po;
        if (!contact_pair(w, pos_in, c, b, s, r, m_b, c2, b2, v2(o.x, o.y), o.z, w.mass[b2], sens_any, off,
                          w.col_off[c2], po))
          return;
        best = k;
        bo = po;
      });
    }
    if (best == ~0ull) break;
    if (bo.pushed) p = add(p, bo.push);
    if (bo.has_corr) p = add(p, bo.corr);
    last = best;
    first = false;
  }
  return p;
}

template <bool MW, bool SPR, bool PEND, bool FUSE>
__global__ void __launch_bounds__(256) k_body_contacts(WorldDev w, const float2* __restrict__ pos_in,
                                                       float2* __restrict__ pos_out, SubstepArgs args) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= w.n_bodies) return;
  const uint32_t c0 = w.body_col_start[b], c1 = w.body_col_start[b + 1];
  float2 p = pos_in[b];
  bool slow = w.bslow[b] != 0;
  if (!slow) {
    Contact list[CONTACT_LIST];
    int nl = 0;
    for (uint32_t qc = c0; qc < c1 && !slow; ++qc) {
      const uint32_t c = w.body_cols[qc];
      const uint32_t n = min((uint32_t)w.ccount[c], CL_CAP);
      if (nl + (int)n > CONTACT_LIST) {
        slow = true;
        break;
      }
      for (uint32_t k = 0; k < n; ++k) list[nl++] = w.clist[(size_t)c * CL_CAP + k];
    }
    if (!slow) {
      sort_contacts(list, nl);
      for (int k = 0; k < nl; ++k) p = add(p, list[k].corr);
    }
  }
  if (slow) {
    // a collider kept only part of its contacts: gather the body's contacts
    // again, or walk them in order on a push-out or a long list
    w.bslow[b] = 0u;
    const WorldParam wp = load_wparam(w, MW ? w.body_world[b] : 0u);
    Contact list[CONTACT_LIST];
    int nl = 0;
    if (collect_contacts(w, wp, pos_in, b, c0, c1, w.mass[b], list, nl)) {
      sort_contacts(list, nl);
      for (int k = 0; k < nl; ++k) p = add(p, list[k].corr);
    } else {
      p = ordered_walk(w, wp, pos_in, b, c0, c1, w.mass[b]);
    }
  }
  if (FUSE) {
    integrate_body<MW, SPR, PEND, false>(w, b, p, pos_out, args);
  } else {
    pos_out[b] = p;
  }
}

// Advances the collision-event substep sequence (after a contact pass).
__global__ void k_ev_tick(WorldDev w) {
  if (threadIdx.x == 0) *w.ev_seq += 1u;
}

void launch_ev_tick(const WorldDev& w, cudaStream_t st) { k_ev_tick<<<1, 32, 0, st>>>(w); }

// Divides a V buffer of displacements by dt in place (storage order).
__global__ void k_v_divide(float2* v, uint32_t n, float dt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = divs(v[i], dt);
}

void launch_v_divide(float2* v, uint32_t n, float dt, cudaStream_t st) {
  if (n) k_v_divide<<<(n + 255u) / 256u, 256, 0, st>>>(v, n, dt);
}

// ---------------------------------------------------------------------------
// One FixedJoint of solve_fixed_joints (physics.rs:430-470), in two parts:
// joint_position moves the two bodies (physics.rs:434-461) and returns the
// anchor difference dp; joint_rotation gives the rotation correction rc of
// physics.rs:462-466 from dp.  Positions never depend on rotations here, so
// the rotation part may run later, as long as each body's rotation receives
// its rc terms in the same order.  The mass terms 1/ma + 1/mb and
// (1/ma) / (1/ma + 1/mb) are constant and come precomputed with the same
// IEEE operations.  joint_position returns false when the joint is skipped
// (anchors closer than 1e-6).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool joint_position(float4 anc, float4 coef, uint32_t loc, float2& pa, float2& pb,
                                               float2& dp) {
  const float2 wa = add(pa, v2(anc.x, anc.y));
  const float2 wb = add(pb, v2(anc.z, anc.w));
  dp = sub(wb, wa);
  const float distance = len2(dp);
  if (distance < 1e-6f) return false;
  const float off_by = distance - coef.z;
  const float2 correction = divs(v2(off_by * dp.x, off_by * dp.y), distance);
  const float ims = coef.x;
  if (loc & JL_STATIC_A) {
    pb = sub(pb, mul(correction, ims));
  } else if (loc & JL_STATIC_B) {
    pa = add(pa, mul(correction, ims));
  } else {
    const float ratio = coef.y;
    pa = add(pa, mul(correction, ratio));
    pb = sub(pb, mul(correction, 1.0f - ratio));
  }
  return true;
}

__device__ __forceinline__ float joint_rotation(float2 dp, float target) {
  const float angle_a = atan2f(dp.y, dp.x);
  const float angle_b = -atan2f(dp.y, -dp.x);  // physics.rs:464 precedence
  return ((angle_b - angle_a) - target) * 0.5f;
}

__device__ __forceinline__ bool fixed_joint(float4 anc, float4 coef, uint32_t loc, float2& pa, float2& pb, float& ra,
                                            float& rb, float dt) {
  float2 dp;
  if (!joint_position(anc, coef, loc, pa, pb, dp)) return false;
  const float rc = joint_rotation(dp, coef.w);
  ra = ra + rc * dt;
  rb = rb - rc * dt;
  return true;
}

// k_joints: one colour of the large components' joints.  Joints of one
// colour touch disjoint bodies, so they run in parallel; colours run in
// sequence, joint_iterations times.
__global__ void __launch_bounds__(256) k_joints(WorldDev w, float2* __restrict__ pos, uint32_t j0, uint32_t j1,
                                                float dt) {
  const uint32_t j = j0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= j1) return;
  const uint32_t ia = w.jnt_a[j], ib = w.jnt_b[j];
  float2 pa = pos[ia], pb = pos[ib];
  float ra = w.rot[ia], rb = w.rot[ib];
  if (!fixed_joint(w.jnt_anc[j], w.jnt_coef[j], w.jnt_local[j], pa, pb, ra, rb, dt)) return;
  pos[ia] = pa;
  pos[ib] = pb;
  w.rot[ia] = ra;
  w.rot[ib] = rb;
  if (!isfinite(ra) || !isfinite(rb)) set_status(w, ST_NAN);
}

// k_joint_blocks: the small components.  A component's joints touch no body
// of another component, so each component runs alone -- all iterations, its
// joints in the reference's arena order -- which gives every body exactly
// the sequence of updates of the reference's sweep.  One thread per
// component; the block's bodies and joints are staged in shared memory.  Up
// to JB_ITERS iterations the sweep runs in three passes, so that the
// sequential chain of a component carries only the position arithmetic:
// (1) per component, the position sweep, keeping every (iteration, joint)
// dp; (2) the rotation corrections of all of them in parallel; (3) per
// component, the rotations summed in the sweep's order.
__global__ void __launch_bounds__(JB_THREADS) k_joint_blocks(WorldDev w, float2* __restrict__ pos, float dt,
                                                             uint32_t iterations) {
  __shared__ float2 s_pos[JB_BODIES];
  __shared__ float s_rot[JB_BODIES];
  __shared__ float4 s_anc[JB_JOINTS];
  __shared__ float4 s_coef[JB_JOINTS];
  __shared__ uint32_t s_loc[JB_JOINTS];
  __shared__ float2 s_dp[JB_ITERS * JB_JOINTS];  // dp of (iteration, joint); then rc in .x
  __shared__ uint8_t s_on[JB_ITERS * JB_JOINTS];  // the joint was applied (not skipped)
  const uint32_t k = blockIdx.x;
  const uint32_t b0 = w.jb_body_start[k], nbody = min(w.jb_body_start[k + 1] - b0, JB_BODIES);
  const uint32_t c0 = w.jb_comp_start[k], c1 = w.jb_comp_start[k + 1];
  const uint32_t qa = w.jb_joint_start[c0], njoint = min(w.jb_joint_start[c1] - qa, JB_JOINTS);
  // staging loops unrolled to their bounds, so that all their loads are in
  // flight together
#pragma unroll
  for (uint32_t r = 0; r < (JB_BODIES + JB_THREADS - 1) / JB_THREADS; ++r) {
    const uint32_t i = threadIdx.x + r * JB_THREADS;
    if (i < nbody) {
      const uint32_t body = w.jb_bodies[b0 + i];
      s_pos[i] = pos[body];
      s_rot[i] = w.rot[body];
    }
  }
#pragma unroll
  for (uint32_t r = 0; r < (JB_JOINTS + JB_THREADS - 1) / JB_THREADS; ++r) {
    const uint32_t i = threadIdx.x + r * JB_THREADS;
    if (i < njoint) {
      s_anc[i] = w.jnt_anc[qa + i];
      s_coef[i] = w.jnt_coef[qa + i];
      s_loc[i] = w.jnt_local[qa + i];
    }
  }
  __syncthreads();
  const uint32_t c = c0 + threadIdx.x;
  const bool mine = c < c1;
  const uint32_t q0 = mine ? w.jb_joint_start[c] - qa : 0u, q1 = mine ? w.jb_joint_start[c + 1] - qa : 0u;
  bool bad = q1 > njoint, nan = false;
  for (uint32_t q = q0; q < q1 && !bad; ++q) {
    const uint32_t loc = s_loc[q];
    bad = (loc & 0x7fffu) >= nbody || ((loc >> 16) & 0x7fffu) >= nbody;
  }
  const bool split = iterations <= JB_ITERS;
  if (mine && !bad) {
    for (uint32_t it = 0; it < iterations; ++it)
      for (uint32_t q = q0; q < q1; ++q) {
        const uint32_t loc = s_loc[q];
        const uint32_t la = loc & 0x7fffu, lb = (loc >> 16) & 0x7fffu;
        float2 pa = s_pos[la], pb = s_pos[lb];
        if (split) {
          float2 dp;
          const bool on = joint_position(s_anc[q], s_coef[q], loc, pa, pb, dp);
          s_dp[it * JB_JOINTS + q] = dp;
          s_on[it * JB_JOINTS + q] = on ? 1 : 0;
          if (!on) continue;
          s_pos[la] = pa;
          s_pos[lb] = pb;
        } else {
          float ra = s_rot[la], rb = s_rot[lb];
          if (!fixed_joint(s_anc[q], s_coef[q], loc, pa, pb, ra, rb, dt)) continue;
          s_pos[la] = pa;
          s_pos[lb] = pb;
          s_rot[la] = ra;
          s_rot[lb] = rb;
          nan = nan || !isfinite(ra) || !isfinite(rb);
        }
      }
  }
  if (split) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < iterations * njoint; i += JB_THREADS) {
      const uint32_t it = i / njoint, q = i - it * njoint, e = it * JB_JOINTS + q;
      if (s_on[e]) s_dp[e].x = joint_rotation(s_dp[e], s_coef[q].w);
    }
    __syncthreads();
    if (mine && !bad) {
      for (uint32_t it = 0; it < iterations; ++it)
        for (uint32_t q = q0; q < q1; ++q) {
          const uint32_t e = it * JB_JOINTS + q;
          if (!s_on[e]) continue;
          const uint32_t loc = s_loc[q];
          const uint32_t la = loc & 0x7fffu, lb = (loc >> 16) & 0x7fffu;
          const float rc = s_dp[e].x;
          const float ra = s_rot[la] + rc * dt;
          const float rb = s_rot[lb] - rc * dt;
          s_rot[la] = ra;
          s_rot[lb] = rb;
          nan = nan || !isfinite(ra) || !isfinite(rb);
        }
    }
  }
  if (mine && bad) set_status(w, ST_BAD_INDEX);
  if (nan) set_status(w, ST_NAN);
  __syncthreads();
#pragma unroll
  for (uint32_t r = 0; r < (JB_BODIES + JB_THREADS - 1) / JB_THREADS; ++r) {
    const uint32_t i = threadIdx.x + r * JB_THREADS;
    if (i < nbody) {
      const uint32_t body = w.jb_bodies[b0 + i];
      pos[body] = s_pos[i];
      w.rot[body] = s_rot[i];
    }
  }
}

template <bool MW, bool SPR, bool PEND, bool SINGLE>
__global__ void __launch_bounds__(256) k_integrate(WorldDev w, const float2* __restrict__ pos_in,
                                                   float2* __restrict__ pos_out, SubstepArgs args) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= w.n_bodies) return;
  integrate_body<MW, SPR, PEND, SINGLE>(w, b, pos_in[b], pos_out, args);
}

// Cell keys and in-cell ranks of every collider from the current snapshots
// (after a load or a host write; in steady state integration records them).
template <bool MW>
__global__ void __launch_bounds__(256) k_keys(WorldDev w) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= w.n_cols) return;
  const WorldParam wp = load_wparam(w, MW ? w.col_world[c] : 0u);
  w.rank[c] = atomicAdd(w.cell_count + cell_key(wp, w.snap[c]), 1u);
}

// ---------------------------------------------------------------------------
// k_emit_pairs: the broadphase output itself.  For every collider (one
// thread per cell-sorted slot) and every candidate in its 3x3 cells with a
// lower collider index, append (hi, lo) -- all candidates (mode 0) or only
// pairs in contact after the reference's filters (mode 1: different parent,
// groups test, dist < ra + rb, physics.rs:249-269).  Pairs past `cap` are
// counted, not written.
// ---------------------------------------------------------------------------
template <bool MW>
__global__ void __launch_bounds__(256) k_emit_pairs(WorldDev w, uint32_t mode, uint32_t* __restrict__ out,
                                                    unsigned long long cap, unsigned long long* __restrict__ count) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= w.n_cols) return;
  const float4 me = w.sorted[e];
  const uint32_t c = __float_as_uint(me.w);
  if (c >= w.n_cols) {
    set_status(w, ST_BAD_INDEX);
    return;
  }
  const float2 s = v2(me.x, me.y);
  const WorldParam wp = load_wparam(w, MW ? w.col_world[c] : 0u);
  for_each_candidate(w, wp, s, [&](uint32_t q) {
    const float4 o = w.sorted[q];
    const uint32_t c2 = __float_as_uint(o.w);
    if (c2 >= c) return;
    if (mode == 1u) {
      if (w.col_parent[c2] == w.col_parent[c]) return;
      const uint32_t m1 = w.col_memb[c], f1 = w.col_filt[c], m2 = w.col_memb[c2], f2 = w.col_filt[c2];
      if (!((m1 & f2) != 0u && (m2 & f1) != 0u)) return;
      const float2 axis = sub(s, v2(o.x, o.y));
      if (!(len2(axis) < (me.z + o.z))) return;
    }
    const unsigned long long k = atomicAdd(count, 1ull);
    if (k < cap) {
      out[2 * k] = c;
      out[2 * k + 1] = c2;
    }
  });
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
static inline uint32_t blocks_for(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

void launch_keys(const WorldDev& w, bool mw, cudaStream_t st) {
  if (!w.n_cols) return;
  const uint32_t g = blocks_for(w.n_cols, 256);
  if (mw) k_keys<true><<<g, 256, 0, st>>>(w);
  else k_keys<false><<<g, 256, 0, st>>>(w);
}

uint32_t launch_scan(const WorldDev& w, cudaStream_t st) {
  const uint32_t tiles = blocks_for(w.n_cells, SCAN_TILE);
  k_tile_sums<<<tiles, SCAN_THREADS, 0, st>>>(w);
  if (tiles > SCAN_PREFIX_TILES && tiles == w.n_tiles) {
    k_tile_prefix<<<1, 1024, 0, st>>>(w);
    k_scan_apply<true><<<tiles, SCAN_THREADS, 0, st>>>(w);
    return 3;
  }
  k_scan_apply<false><<<tiles, SCAN_THREADS, 0, st>>>(w);
  return 2;
}

#define BLOBS_DISPATCH_BOOL(v, NAME, ...) \
  if (v) {                                \
    constexpr bool NAME = true;           \
    __VA_ARGS__;                          \
  } else {                                \
    constexpr bool NAME = false;          \
    __VA_ARGS__;                          \
  }

void launch_scatter_forces(const WorldDev& w, const float2* pos, bool mw, bool scatter, bool springs, bool pending,
                           cudaStream_t st) {
  const uint32_t nc = scatter ? w.n_cols : 0u, nb = springs ? w.n_bodies : 0u;
  const uint32_t n = nc > nb ? nc : nb;
  if (!n) return;
  const uint32_t g = blocks_for(n, 256);
  BLOBS_DISPATCH_BOOL(mw, MW,
    BLOBS_DISPATCH_BOOL(scatter, SC,
      BLOBS_DISPATCH_BOOL(springs, SP,
        BLOBS_DISPATCH_BOOL(pending, PE, k_scatter_forces<MW, SC, SP, PE><<<g, 256, 0, st>>>(w, pos)))));
}

uint32_t launch_contacts(const WorldDev& w, const float2* pos_in, float2* pos_out, bool mw, bool single, bool springs,
                     bool pending, bool fuse, float dt, float old_dt, bool do_keys, bool rot_dynamic,
                     cudaStream_t st) {
  SubstepArgs a{dt, old_dt, dt / old_dt, dt / dt, do_keys ? 1u : 0u, rot_dynamic ? 1u : 0u};
  if (single) {
    if (!w.n_cols) return 0u;
    const uint32_t g = blocks_for(w.n_cols, 256);
    BLOBS_DISPATCH_BOOL(mw, MW,
      BLOBS_DISPATCH_BOOL(springs, SP,
        BLOBS_DISPATCH_BOOL(pending, PE,
          BLOBS_DISPATCH_BOOL(fuse, FU, k_contact_single<MW, SP, PE, FU><<<g, 256, 0, st>>>(w, pos_in, pos_out, a)))));
  } else {
    if (!w.n_bodies) return 0u;
    if (w.n_cols) {
      const uint32_t gc = blocks_for(w.n_cols, 256);
      BLOBS_DISPATCH_BOOL(mw, MW, k_collider_contacts<MW><<<gc, 256, 0, st>>>(w, pos_in));
    }
    const uint32_t g = blocks_for(w.n_bodies, 256);
    BLOBS_DISPATCH_BOOL(mw, MW,
      BLOBS_DISPATCH_BOOL(springs, SP,
        BLOBS_DISPATCH_BOOL(pending, PE,
          BLOBS_DISPATCH_BOOL(fuse, FU, k_body_contacts<MW, SP, PE, FU><<<g, 256, 0, st>>>(w, pos_in, pos_out, a)))));
    return w.n_cols ? 2u : 1u;
  }
  return 1u;
}

void launch_joint_blocks(const WorldDev& w, float2* pos, float dt, uint32_t iterations, cudaStream_t st) {
  if (!w.n_jblocks) return;
  k_joint_blocks<<<w.n_jblocks, JB_THREADS, 0, st>>>(w, pos, dt, iterations);
}

void launch_joints(const WorldDev& w, float2* pos, uint32_t j0, uint32_t j1, float dt, cudaStream_t st) {
  if (j1 <= j0) return;
  k_joints<<<blocks_for(j1 - j0, 256), 256, 0, st>>>(w, pos, j0, j1, dt);
}

void launch_integrate(const WorldDev& w, const float2* pos_in, float2* pos_out, bool mw, bool single, bool springs,
                      bool pending, float dt, float old_dt, bool do_keys, bool rot_dynamic, cudaStream_t st) {
  if (!w.n_bodies) return;
  SubstepArgs a{dt, old_dt, dt / old_dt, dt / dt, do_keys ? 1u : 0u, rot_dynamic ? 1u : 0u};
  const uint32_t g = blocks_for(w.n_bodies, 256);
  BLOBS_DISPATCH_BOOL(mw, MW,
    BLOBS_DISPATCH_BOOL(springs, SP,
      BLOBS_DISPATCH_BOOL(pending, PE,
        BLOBS_DISPATCH_BOOL(single, SI, k_integrate<MW, SP, PE, SI><<<g, 256, 0, st>>>(w, pos_in, pos_out, a)))));
}

void launch_emit_pairs(const WorldDev& w, bool mw, uint32_t mode, uint32_t* out, unsigned long long cap,
                       unsigned long long* count, cudaStream_t st) {
  if (!w.n_cols) return;
  const uint32_t g = blocks_for(w.n_cols, 256);
  if (mw) k_emit_pairs<true><<<g, 256, 0, st>>>(w, mode, out, cap, count);
  else k_emit_pairs<false><<<g, 256, 0, st>>>(w, mode, out, cap, count);
}

}  // namespace blobs
