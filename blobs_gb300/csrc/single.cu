// single.cu -- the single-sphere path: every body owns exactly one collider
// at offset zero with default groups and no sensor, and there are no fixed
// joints (configurations 1, 2, 4 and 5).  Body state lives in cell-sorted
// storage order, so the contact gather and the integration read and write
// it coalesced:
//
//   k_permute      storage slot i of the previous substep -> slot
//                  cell_start[key] + rank of this substep (counting-sort
//                  scatter of the whole body record; bodies move little per
//                  substep, so the writes are nearly coalesced)
//   k_step_single  per slot: gravity + springs, contacts over the 3x3 cells
//                  applied in the reference's pair order, Verlet
//                  integration, constraints, and the cell key / rank of the
//                  next substep
//
// Records: A = (snapshot x, snapshot y, radius, arena id bits),
//          B = (position x, y, position_old x, y), V = calculated_velocity,
//          body_c[id] = (mass, gravity_mod, bounding radius, flags | world << 8).
// Compiled with --fmad=false (see device.cuh).
#include "device.cuh"
#include "kernels.h"

namespace blobs {

namespace {

__device__ __forceinline__ uint32_t rec_flags(float4 c) { return __float_as_uint(c.w) & 0xffu; }
__device__ __forceinline__ uint32_t rec_world(float4 c) { return __float_as_uint(c.w) >> 8; }

// The cell-sorted slots of the 3 rows of 3 cells around point s: up to six
// contiguous segments (a row splits in two where the torus wraps).
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

// Slot of the t-th candidate of the segments (t < total).
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

// Visit every slot of the segments in one flattened loop (less divergence
// than a loop per row).
template <class F>
__device__ __forceinline__ void visit(const Segments& g, F&& f) {
  const uint32_t total = g.l[0] + g.l[1] + g.l[2] + g.l[3] + g.l[4] + g.l[5];
  uint32_t seg = 0, q = g.s[0], left = g.l[0];
  for (uint32_t t = 0; t < total; ++t) {
    while (left == 0u) {
      ++seg;
      switch (seg) {
        case 1: q = g.s[1]; left = g.l[1]; break;
        case 2: q = g.s[2]; left = g.l[2]; break;
        case 3: q = g.s[3]; left = g.l[3]; break;
        case 4: q = g.s[4]; left = g.l[4]; break;
        default: q = g.s[5]; left = g.l[5]; break;
      }
    }
    f(q);
    ++q;
    --left;
  }
}

// Exact contact test of the reference (physics.rs:264-269): sqrt(d.d) < ra + rb.
// A squared-distance test rejects first: T >= (ra + rb)^2 strictly, so
// d.d > T implies sqrt(d.d) >= ra + rb and the reference rejects too.
__device__ __forceinline__ bool near_pair(float dx, float dy, float mind, float& D) {
  D = (dx * dx) + (dy * dy);
  const float T = (mind * mind) * 1.00000024f;
  return !(D > T);
}

struct SinglePair {
  float2 corr;
  float2 push;
  bool pushed;
};

// One contact of body `c` (at p, snapshot s, radius r, mass m) with body c2
// (snapshot s2, radius r2): the increment to c's position.  Returns false if
// not in contact.  Push-out (physics.rs:272-286) uses positions at the start
// of the contact pass.
__device__ __forceinline__ bool single_pair(const WorldDev& w, uint32_t c, float2 p, float2 s, float r, float m,
                                            uint32_t c2, const float4* __restrict__ B, uint32_t q, float2 s2,
                                            float r2, SinglePair& out) {
  const float dx = s.x - s2.x, dy = s.y - s2.y;
  float D;
  const float mind = r + r2;
  if (!near_pair(dx, dy, mind, D)) return false;
  float d = sqrtf(D);
  if (!(d < mind)) return false;
  const bool hi = c > c2;
  float2 axis = hi ? v2(dx, dy) : v2(-dx, -dy);
  out.pushed = false;
  out.push = v2(0.0f, 0.0f);
  if (d < 1e-6f) {
    const float2 p2 = v2(B[q].x, B[q].y);
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
  const float m2 = w.body_c[c2].x;
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

__device__ __forceinline__ void count_warp(const WorldDev& w, uint32_t ncontacts, uint32_t npush) {
  uint32_t t = ncontacts, p = npush;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_xor_sync(0xffffffffu, t, o);
    p += __shfl_xor_sync(0xffffffffu, p, o);
  }
  if ((threadIdx.x & 31u) == 0u) {
    const uint32_t bin = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) & (COUNTER_BINS - 1);
    if (t) {
      atomicAdd(w.contacts_total + bin, (unsigned long long)t);
      atomicAdd(w.contacts_sub + bin, t);
    }
    if (p) atomicAdd(w.pushouts_total + bin, (unsigned long long)p);
  }
}


}  // namespace

template <bool SPR>
__global__ void __launch_bounds__(256) k_permute(WorldDev w, const float4* __restrict__ a_in,
                                                 const float4* __restrict__ b_in, const float2* __restrict__ v_in,
                                                 float4* __restrict__ a_out, float4* __restrict__ b_out,
                                                 float2* __restrict__ v_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n_bodies) return;
  const uint32_t key = w.key[i];
  const uint32_t j = w.cell_start[key] + w.rank[i];
  if (j >= w.n_bodies) {
    atomicOr(w.status, ST_BAD_INDEX);
    return;
  }
  const float4 a = a_in[i];
  a_out[j] = a;
  b_out[j] = b_in[i];
  w.ckey[j] = key;
  if (SPR) {
    v_out[j] = v_in[i];
    const uint32_t id = __float_as_uint(a.w);
    if (id < w.n_bodies) w.where[id] = j;
  }
}

template <bool MW, bool SPR, bool PEND, bool CONTACTS>
__global__ void __launch_bounds__(256) k_step_single(WorldDev w, const float4* __restrict__ A,
                                                     const float4* __restrict__ B, const float2* __restrict__ V,
                                                     float4* __restrict__ a_out, float4* __restrict__ b_out,
                                                     float2* __restrict__ v_out, SubstepArgs args) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t ncontacts = 0, npush = 0;
  if (j < w.n_bodies) {
    const float4 a = A[j];
    const float4 b = B[j];
    uint32_t c = __float_as_uint(a.w);
    if (c >= w.n_bodies) {
      atomicOr(w.status, ST_BAD_INDEX);
      c = 0;
    }
    const float4 rec = w.body_c[c];
    const float m = rec.x;
    const uint32_t fl = rec_flags(rec);
    const WorldParam wp = w.wparam[MW ? rec_world(rec) : 0u];
    const float2 s = v2(a.x, a.y);
    const float r = a.z;
    const float2 p0 = v2(b.x, b.y);  // position at the start of the substep
    float2 p = p0;

    if (CONTACTS) {
      const Segments g = segments(w, wp, w.ckey[j]);
      const uint32_t total = g.l[0] + g.l[1] + g.l[2] + g.l[3] + g.l[4] + g.l[5];
      if (total <= 64u) {
        // Phase 1: one squared-distance test per candidate; near candidates
        // become bits of their position in the 3x3 enumeration.
        unsigned long long near = 0ull;
        uint32_t t = 0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const uint32_t q1 = g.s[k] + g.l[k];
          for (uint32_t q = g.s[k]; q < q1; ++q, ++t) {
            const float4 o = A[q];
            const float dx = s.x - o.x, dy = s.y - o.y;
            float D;
            if (near_pair(dx, dy, r + o.z, D) && q != j) near |= 1ull << t;
          }
        }
        // Phase 2: apply the near candidates in ascending neighbour id (the
        // reference's pair order for this body), smallest id first.
        while (near) {
          unsigned long long best_bit = 0ull;
          uint32_t best = 0xffffffffu, bq = 0u;
          float4 bo = make_float4(0.f, 0.f, 0.f, 0.f);
          for (unsigned long long mk = near; mk; mk &= mk - 1ull) {
            const uint32_t tt = (uint32_t)(__ffsll((long long)mk) - 1);
            const uint32_t q = slot_of(g, tt);
            const float4 o = A[q];
            const uint32_t c2 = __float_as_uint(o.w);
            if (c2 < best) {
              best = c2;
              bq = q;
              bo = o;
              best_bit = mk & (~mk + 1ull);
            }
          }
          near &= ~best_bit;
          if (best >= w.n_bodies) continue;
          SinglePair sp;
          if (!single_pair(w, c, p0, s, r, m, best, B, bq, v2(bo.x, bo.y), bo.z, sp)) continue;
          if (sp.pushed) p = add(p, sp.push);
          p = add(p, sp.corr);
          if (best < c) {
            ++ncontacts;
            npush += sp.pushed ? 1u : 0u;
          }
        }
      } else {
        // more than 64 candidates: exact selection walk over all of them
        uint32_t last = 0u;
        bool first = true;
        while (true) {
          uint32_t best = 0xffffffffu;
          SinglePair bo;
          bool found = false;
          visit(g, [&](uint32_t q) {
            if (q == j) return;
            const float4 o = A[q];
            const uint32_t c2 = __float_as_uint(o.w);
            if (c2 >= w.n_bodies || (!first && c2 <= last) || (found && c2 >= best)) return;
            SinglePair sp;
            if (!single_pair(w, c, p0, s, r, m, c2, B, q, v2(o.x, o.y), o.z, sp)) return;
            best = c2;
            bo = sp;
            found = true;
          });
          if (!found) break;
          if (bo.pushed) p = add(p, bo.push);
          p = add(p, bo.corr);
          if (best < c) {
            ++ncontacts;
            npush += bo.pushed ? 1u : 0u;
          }
          last = best;
          first = false;
        }
      }
    }

    // ---- update_objects (physics.rs:323-367) with gravity + springs ----
    const float dt = args.dt;
    float2 po, vel;
    if (fl & BF_STATIC) {
      po = p;
      vel = v2(0.0f, 0.0f);
    } else {
      po = v2(b.z, b.w);
      if (PEND && (fl & BF_VREQ)) po = sub(p, mul(w.vreq[c], dt));
      const float ratio = (fl & BF_FIRST_DYN) ? args.ratio_first : args.ratio_rest;
      const float2 disp = mul(sub(p, po), ratio);
      float2 acc = PEND ? w.pend_acc[c] : v2(0.0f, 0.0f);
      acc = add(acc, mul(w.gravity, rec.y));
      if (SPR) {
        const uint32_t q0 = w.body_spr_start[c], q1 = w.body_spr_start[c + 1];
        for (uint32_t qq = q0; qq < q1; ++qq) {
          const uint32_t e = w.body_spr[qq];
          const uint32_t sidx = e >> 1;
          const uint32_t ia = w.spr_a[sidx], ib = w.spr_b[sidx];
          const uint32_t other = (e & 1u) ? ia : ib;
          const uint32_t so = w.where[other];
          const float2 po_pos = v2(B[so].x, B[so].y);
          const float2 po_vel = V[so];
          const float2 va = (e & 1u) ? po_vel : V[j], vb = (e & 1u) ? V[j] : po_vel;
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
          acc = add(acc, divs(f, m));
        }
      }
      po = p;
      p = add(p, add(disp, mul(mul(acc, dt), dt)));
      if (args.rot_dynamic) {
        const float tq = PEND ? w.pend_torque[c] : 0.0f;
        float av = w.angvel[c];
        av = av + (tq / w.inertia[c]) * dt;
        w.angvel[c] = av;
        w.rot[c] = w.rot[c] + av * dt;
      }
      // calculated_velocity = disp / dt (physics.rs:357).  Without springs
      // nothing reads it during the step: keep disp and divide on read.
      vel = SPR ? divs(disp, dt) : disp;
    }
    const float2 snap = v2(0.0f + p.x, 0.0f + p.y);  // rot(theta) * 0 + p
    for (uint32_t k = 0; k < w.n_circles; ++k) {
      const float2 cc = v2(w.circles[3 * k], w.circles[3 * k + 1]);
      const float radius = w.circles[3 * k + 2];
      const float2 to = sub(p, cc);
      const float dist = len2(to);
      if (dist > radius) p = add(cc, mul(divs(to, dist), radius));
    }
    if (wp.has_box) {
      const float br = rec.z;
      p.x = fminf(fmaxf(p.x, wp.box_lo_x + br), wp.box_hi_x - br);
      p.y = fminf(fmaxf(p.y, wp.box_lo_y + br), wp.box_hi_y - br);
    }
    a_out[j] = make_float4(snap.x, snap.y, r, a.w);
    b_out[j] = make_float4(p.x, p.y, po.x, po.y);
    v_out[j] = vel;
    if (args.do_keys) {
      const uint32_t key = cell_key(wp, snap);
      w.key[j] = key;
      w.rank[j] = atomicAdd(w.cell_count + key, 1u);
    }
  }
  if (CONTACTS) count_warp(w, ncontacts, npush);
}

// Keys and ranks of the current storage (after a load or a host write).
template <bool MW>
__global__ void __launch_bounds__(256) k_keys_single(WorldDev w, const float4* __restrict__ A) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= w.n_bodies) return;
  const float4 a = A[j];
  const uint32_t c = __float_as_uint(a.w);
  const WorldParam wp = w.wparam[MW ? rec_world(w.body_c[c < w.n_bodies ? c : 0u]) : 0u];
  const uint32_t key = cell_key(wp, v2(a.x, a.y));
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
    const float2 v = V[j];
    // V holds the displacement of the last substep when v_div != 0 (static
    // bodies store 0, and 0 / dt = 0)
    vel[c] = v_div != 0.0f ? divs(v, v_div) : v;
  }
  if (snap) snap[c] = v2(a.x, a.y);
}

__global__ void __launch_bounds__(256) k_write_single(WorldDev w, const float4* __restrict__ A, float4* B,
                                                      float2* V, const float2* pos, const float2* pos_old,
                                                      const float2* vel) {
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
}

__global__ void __launch_bounds__(256) k_where_single(WorldDev w, const float4* __restrict__ A) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= w.n_bodies) return;
  const uint32_t c = __float_as_uint(A[j].w);
  if (c < w.n_bodies) w.where[c] = j;
}

// ---------------------------------------------------------------------------
static inline uint32_t nblocks(uint32_t n) { return (n + 255u) / 256u; }

void launch_permute(const WorldDev& w, int from, bool springs, cudaStream_t st) {
  if (!w.n_bodies) return;
  const int to = from ^ 1;
  if (springs)
    k_permute<true><<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[from], w.sb[from], w.sv[from], w.sa[to], w.sb[to],
                                                         w.sv[to]);
  else
    k_permute<false><<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[from], w.sb[from], w.sv[from], w.sa[to],
                                                          w.sb[to], w.sv[to]);
}

#define BLOBS_B(v, NAME, ...) \
  if (v) {                    \
    constexpr bool NAME = true; \
    __VA_ARGS__;              \
  } else {                    \
    constexpr bool NAME = false; \
    __VA_ARGS__;              \
  }

void launch_step_single(const WorldDev& w, int from, int to, bool mw, bool springs, bool pending, bool contacts,
                        float dt, float old_dt, bool do_keys, bool rot_dynamic, cudaStream_t st) {
  if (!w.n_bodies) return;
  SubstepArgs a{dt, old_dt, dt / old_dt, dt / dt, do_keys ? 1u : 0u, rot_dynamic ? 1u : 0u};
  const uint32_t g = nblocks(w.n_bodies);
  BLOBS_B(mw, MW,
    BLOBS_B(springs, SP,
      BLOBS_B(pending, PE,
        BLOBS_B(contacts, CO,
          k_step_single<MW, SP, PE, CO><<<g, 256, 0, st>>>(w, w.sa[from], w.sb[from], w.sv[from], w.sa[to],
                                                          w.sb[to], w.sv[to], a)))));
}

void launch_keys_single(const WorldDev& w, int cur, bool mw, cudaStream_t st) {
  if (!w.n_bodies) return;
  if (mw) k_keys_single<true><<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[cur]);
  else k_keys_single<false><<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[cur]);
}

void launch_gather_single(const WorldDev& w, int cur, float2* pos, float2* pos_old, float2* vel, float2* snap,
                          float v_div, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_gather_single<<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[cur], w.sb[cur], w.sv[cur], pos, pos_old, vel, snap,
                                                       v_div);
}

void launch_write_single(const WorldDev& w, int cur, const float2* pos, const float2* pos_old, const float2* vel,
                         cudaStream_t st) {
  if (!w.n_bodies) return;
  k_write_single<<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[cur], w.sb[cur], w.sv[cur], pos, pos_old, vel);
}

void launch_where_single(const WorldDev& w, int cur, cudaStream_t st) {
  if (!w.n_bodies) return;
  k_where_single<<<nblocks(w.n_bodies), 256, 0, st>>>(w, w.sa[cur]);
}

}  // namespace blobs
