// device.cuh -- device-side world layout and the f32 arithmetic of the blobs
// step (darthdeus/blobs 0.2.1, blobs/src/physics.rs), shared by every kernel.
//
// Every translation unit that includes this file is compiled with
// --fmad=false: the reference never contracts a*b+c into an FMA (Rust does
// not contract, glam's Vec2 is scalar code), and the contact / spring /
// integration results are bit-exact only if the GPU rounds every product and
// sum separately, in the same order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace blobs {

// Per-body flag bits.
enum : uint8_t {
  BF_STATIC = 1,     // RigidBodyType::Static (rigid_body.rs:211-213)
  BF_FIRST_DYN = 2,  // first non-static body of its world in arena order: sees dt/old_dt (physics.rs:338-339)
  BF_VREQ = 4,       // velocity_request is Some (consumed by the next substep, physics.rs:334-336)
};

// Device status bits, read back by the host after a synchronising call.
enum : uint32_t {
  ST_NAN = 1u,         // NaN contact normal or non-finite rotation (physics.rs:293, 471-474)
  ST_TIMEOUT = 2u,     // a bounded spin-wait gave up (reserved: no kernel waits on another)
  ST_BAD_INDEX = 4u,   // a device bounds check fired
};

// Per-world parameters (a batch packs many independent worlds).
struct WorldParam {
  uint32_t cell_base;   // first cell of this world's toroidal grid in the global cell table
  uint32_t log2w;       // grid is (1 << log2w) x (1 << log2h) cells, coordinates wrap
  uint32_t log2h;
  float cs;             // cell edge
  float box_lo_x, box_lo_y, box_hi_x, box_hi_y;
  uint32_t has_box;     // axis-aligned wall extension enabled
  float inv_cs;         // 1 / cs (rounded once, on the host)
  uint32_t first_dyn;   // arena id of the world's first non-static body (uniform single-sphere worlds)
  float uniform_gmod;   // gravity_mod shared by every body (uniform single-sphere worlds)
  float ox, oy;         // grid origin: the world's extent maps to cells 1 .. W-2, away from the wrap
  uint32_t pad[2];
};

// One contact as seen from one body: its place in the reference's pair
// sequence and the body's position increment.
struct Contact {
  unsigned long long key;  // (hi << 33) | (lo << 1), hi > lo collider indices
  float2 corr;             // signed position increment for this body
};

// Every device pointer of a loaded scene.  Passed to kernels by value.
struct WorldDev {
  uint32_t n_bodies, n_cols, n_springs, n_joints, n_worlds, n_circles, n_cells, n_tiles;
  float2 gravity;

  // bodies (arena order)
  float2* pos_old;
  float2* vel;          // calculated_velocity
  float2* acc;          // per-substep force accumulator (springs present)
  float* rot;
  float* angvel;
  float* mass;          // calculated_mass (rigid_body.rs:96-128)
  float* inertia;
  float* gmod;          // gravity_mod
  float* bound_r;       // bounding radius for the wall extension
  uint8_t* bflags;
  float2* pend_acc;     // acceleration present before the step (consumed by its first substep)
  float* pend_torque;
  float2* vreq;
  uint32_t* body_world;      // batched only
  uint32_t* body_col_start;  // n_bodies + 1: colliders of a body (ascending)
  uint32_t* body_cols;
  uint32_t* body_spr_start;  // n_bodies + 1: incident springs, ascending spring index
  uint32_t* body_spr;        // (spring index << 1) | (1 if the body is endpoint b)

  // colliders (arena order)
  uint32_t* col_parent;
  float2* col_off;
  float* col_radius;
  uint32_t* col_memb;
  uint32_t* col_filt;
  uint8_t* col_sensor;
  float2* snap;              // absolute_transform.translation
  uint32_t* col_world;       // batched only

  // springs (arena order)
  uint32_t* spr_a;
  uint32_t* spr_b;
  float* spr_rest;
  float* spr_k;
  float* spr_c;

  // joints, stored in the processing order: first the joints of the small
  // components, component by component (arena order inside each), then the
  // joints of the large components in (colour, arena index) order
  uint32_t* jnt_a;
  uint32_t* jnt_b;
  float4* jnt_anc;           // (anchor_a, anchor_b)
  float4* jnt_coef;          // (1/ma + 1/mb, (1/ma) / that, distance, target_angle), from the constant masses
  uint32_t* jnt_local;       // block-local body slots a | b << 16 (small components) | JL_STATIC_A / _B
  // small components, solved in shared memory by k_joint_blocks: block k
  // holds components [jb_comp_start[k], jb_comp_start[k+1]) and the bodies
  // jb_bodies[jb_body_start[k] .. jb_body_start[k+1]); component c is the
  // joints [jb_joint_start[c], jb_joint_start[c+1]) of the processing order
  uint32_t* jb_comp_start;
  uint32_t* jb_joint_start;
  uint32_t* jb_body_start;
  uint32_t* jb_bodies;
  uint32_t n_jblocks;

  float* circles;            // 3 per circle
  WorldParam* wparam;

  // broadphase
  uint32_t* cell_count;      // n_cells, zero between substeps
  uint32_t* cell_start;      // n_cells + 1
  uint32_t* rank;            // per collider: slot inside its cell
  float4* sorted;            // per slot: (x, y, radius, collider index bits)
  Contact* clist;            // general path, per collider: up to CL_CAP contacts of the substep
  uint8_t* ccount;           // general path, per collider: contacts in clist
  uint8_t* bslow;            // general path, per body: contacts need the ordered walk (zero between substeps)
  uint32_t* tile_sums;       // per scan tile

  // single-sphere path: body storage re-sorted into cell order once per step
  float4* sa[2];             // (snapshot x, y, radius, arena id bits), double-buffered per substep
  float4* sb[2];             // (position x, y, position_old x, y)
  float2* sv[2];             // calculated_velocity (or the last substep's displacement)
  float4* cand;              // cell-order copy of sa: the candidate records of a substep
  float4* body_c;            // arena order: (mass, gravity_mod, bounding radius, flags | world << 8)
  uint32_t* key;             // per storage slot: cell of the snapshot for the next substep
  uint32_t* ckey;            // per storage slot: cell the permute sorted the body into
  uint32_t* where;           // arena id -> storage slot
  uint32_t* defer_list;      // storage slots whose substep k_step_deferred finishes (plain steps)
  uint32_t* defer_count;     // entries of defer_list this substep (zeroed by the cell scan)

  // collision event stream (NULL when off): one record per resolved pair,
  // appended in any order and put in the reference's order on the host by
  // (substep sequence, a, b)
  uint4* ev_rec;             // (sequence, collider a, collider b, 0), a > b
  float4* ev_vel;            // (impact_vel_a, impact_vel_b): calculated_velocity of the parents
  uint32_t* ev_count;        // appended so far (may exceed ev_cap: overflow)
  uint32_t* ev_seq;          // substep sequence number, advanced after each contact pass
  uint32_t ev_cap;

  // counters, each spread over COUNTER_BINS bins that the host sums
  unsigned long long* contacts_total;
  unsigned long long* pushouts_total;
  uint32_t* contacts_sub;    // contacts of the most recent substep
  unsigned long long* defer_total;  // bodies deferred to a warp each (many candidates or near candidates)
  uint32_t* defer_sub;       // the same in the most recent substep
  uint32_t* status;
};

// ---------------------------------------------------------------------------
// glam Vec2 arithmetic, one rounding per operation.
// ---------------------------------------------------------------------------
__device__ __host__ __forceinline__ float2 v2(float x, float y) { return make_float2(x, y); }
__device__ __host__ __forceinline__ float2 add(float2 a, float2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __host__ __forceinline__ float2 sub(float2 a, float2 b) { return v2(a.x - b.x, a.y - b.y); }
__device__ __host__ __forceinline__ float2 mul(float2 a, float s) { return v2(a.x * s, a.y * s); }
__device__ __host__ __forceinline__ float2 mulv(float2 a, float2 b) { return v2(a.x * b.x, a.y * b.y); }
__device__ __host__ __forceinline__ float2 divs(float2 a, float s) { return v2(a.x / s, a.y / s); }
__device__ __host__ __forceinline__ float dot2(float2 a, float2 b) { return (a.x * b.x) + (a.y * b.y); }
__device__ __host__ __forceinline__ float len2(float2 a) { return sqrtf(dot2(a, a)); }

// Pre-test of the reference's contact test (physics.rs:264-269),
// sqrt(d.d) < ra + rb, without the square root: T >= (ra + rb)^2 strictly,
// so d.d > T implies sqrt(d.d) >= ra + rb and the reference rejects too.
__device__ __host__ __forceinline__ bool near_pair(float dx, float dy, float mind) {
  const float D = (dx * dx) + (dy * dy);
  const float T = (mind * mind) * 1.00000024f;
  return !(D > T);
}

// Rust `(v / cs).floor() as i32`: IEEE division, saturating conversion, NaN -> 0
// (spatial.rs:57-62 semantics).
__device__ __host__ __forceinline__ int32_t cell_coord(float v, float cs) {
  float q = floorf(v / cs);
  if (q != q) return 0;
  if (q >= 2147483648.0f) return 2147483647;
  if (q <= -2147483648.0f) return (-2147483647 - 1);
  return (int32_t)q;
}

// floor(q) as int32, saturating, NaN -> 0.
__device__ __host__ __forceinline__ int32_t floor_sat(float q) {
#ifdef __CUDA_ARCH__
  // cvt.rmi.s32.f32: floor, saturating, NaN -> 0 -- the same function
  return __float2int_rd(q);
#else
  q = floorf(q);
  if (q != q) return 0;
  if (q >= 2147483648.0f) return 2147483647;
  if (q <= -2147483648.0f) return (-2147483647 - 1);
  return (int32_t)q;
#endif
}

// Below this many cells from the grid origin the plain f32 formula is used.
constexpr float GRID_FAST_CELLS = 32768.0f;

// floor((v - o) * inv) in real arithmetic, for |v - o| * inv at or beyond
// GRID_FAST_CELLS: the difference is carried exactly as s + e (TwoSum), the
// product s * inv exactly as p + r1 (an FMA residual, exact in f32), so the
// result is within ~|X| 2^-46 cells of the real-number floor for every
// |X| < 2^31 (saturating beyond, which merges cells and stays exact).
__device__ __host__ __noinline__ inline int32_t grid_coord_far(float v, float o, float inv) {
  const float s = v - o;
  const float bb = s - v;
  const float e = (v - (s - bb)) + ((-o) - bb);
  const float p = s * inv;
  const float r1 = fmaf(s, inv, -p);
  const float t = r1 + e * inv;
  const float fl = floorf(p);
  float fg = floorf((p - fl) + t);  // p - floor(p) is exact
  fg = fminf(fmaxf(fg, -1024.0f), 1024.0f);
  const float flc = fminf(fmaxf(fl, -4.0e18f), 4.0e18f);  // saturate after the sum, in 64 bits
  const long long k = (long long)flc + (long long)fg;
  return k > 2147483647ll ? 2147483647 : (k < -2147483648ll ? (int32_t)(-2147483647 - 1) : (int32_t)k);
}

// Cell coordinate of the broadphase grid: floor((v - o) * inv), saturating,
// NaN -> 0, monotone in v.  With cs >= 2 rmax (1 + 1/64) and inv = fl(1/cs)
// two spheres in contact under the reference's own f32 test
// (sqrt(d.d) < ra + rb) are less than 0.985 of a grid cell apart; the
// plain formula fl(fl(v - o) * inv) is off by at most 2^-8 of a cell below
// GRID_FAST_CELLS cells from the origin, and grid_coord_far is off by a
// negligible amount above it, so such spheres always land in
// 3x3-neighbouring cells, however far from the origin they are.
__device__ __host__ __forceinline__ int32_t grid_coord(float v, float o, float inv) {
  const float q = (v - o) * inv;
  const float aq = fabsf(q);
  if (aq < GRID_FAST_CELLS || !(aq <= 3.402823466e38f)) return floor_sat(q);  // NaN, +-inf: saturate
  return grid_coord_far(v, o, inv);
}

// Global cell index of a point in world `wp`'s toroidal grid:
// cell = floor((v - origin) * (1/cs)) wrapped mod the grid size.
__device__ __host__ __forceinline__ uint32_t cell_key(const WorldParam& wp, float2 s) {
  uint32_t ix = (uint32_t)grid_coord(s.x, wp.ox, wp.inv_cs) & ((1u << wp.log2w) - 1u);
  uint32_t iy = (uint32_t)grid_coord(s.y, wp.oy, wp.inv_cs) & ((1u << wp.log2h) - 1u);
  return wp.cell_base + ((iy << wp.log2w) | ix);
}

// Affine2::from_angle_translation(rot, pos) * offset -> translation
// (rigid_body.rs:88-90, physics.rs:360-366; glam Mat2 * Vec2 column form).
__device__ __forceinline__ float2 collider_translation(float rot, float2 pos, float2 off) {
  float s, c;
  sincosf(rot, &s, &c);
  float2 m = v2((c * off.x) + ((-s) * off.y), (s * off.x) + (c * off.y));
  return add(m, pos);
}

// Per-substep scalars of the integration.
struct SubstepArgs {
  float dt;
  float old_dt;
  float ratio_first;     // dt / old_dt, the first non-static body's factor (physics.rs:338)
  float ratio_rest;      // dt / dt (exactly 1 for a finite non-zero dt)
  uint32_t do_keys;
  uint32_t rot_dynamic;  // 0: every angular velocity is 0 and no torque is pending -> rotation is constant
};

// Launch arguments of the single-sphere kernels.
struct SingleArgs {
  const float4* a_in;
  const float4* b_in;
  const float2* v_in;
  float4* a_out;
  float4* b_out;
  float2* v_out;
  const float4* cand;        // candidate records in cell order
  const uint32_t* own_cell;  // cell of each storage slot in this substep's order
  float dt, ratio_first, ratio_rest;
  uint32_t contacts, pending, springs, rot_dynamic, do_keys, write_v, move_v;
  uint32_t v_vel;            // V holds calculated_velocity (else the displacement of the last substep)
  uint32_t mass4r;           // every body's mass is 4 x its radius: a partner's mass follows from its candidate record
  // contact recording for the adjoint (NULL in ordinary steps): every
  // contact of body c in the order it was applied (ascending partner id),
  // rec_list[k * n_bodies + c] = partner | pushed << 31 for k < REC_CAP,
  // rec_n[c] = the number of contacts (more than REC_CAP: overflow),
  // *rec_max = the largest rec_n of the substep
  uint32_t* rec_list;
  uint32_t* rec_n;
  uint32_t* rec_max;
};

// Append one collision event (physics.rs:304-311): the pair (a, b) with
// a > b in collider order and the parents' calculated_velocity at the start
// of the contact pass.
// The lanes of a warp that append together take their slots with one atomic
// (the buffer is put in order on the host, so any order of slots will do).
__device__ __forceinline__ void record_event(const WorldDev& w, uint32_t a, uint32_t b, float2 va, float2 vb) {
  const uint32_t active = __activemask();
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t leader = (uint32_t)(__ffs(active) - 1);
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(w.ev_count, (uint32_t)__popc(active));
  base = __shfl_sync(active, base, leader);
  const uint32_t k = base + (uint32_t)__popc(active & ((1u << lane) - 1u));
  if (k < w.ev_cap) {
    w.ev_rec[k] = make_uint4(*w.ev_seq, a, b, 0u);
    w.ev_vel[k] = make_float4(va.x, va.y, vb.x, vb.y);
  }
}

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr uint32_t SCAN_PREFIX_TILES = 256;  // more tiles: their prefix by one k_tile_prefix block
constexpr int CONTACT_LIST = 24;           // per-body sorted contact list kept in registers
constexpr uint32_t CL_CAP = 8;             // general path: contacts kept per collider
constexpr uint32_t COUNTER_BINS = 64;
constexpr uint32_t REC_CAP = 16;           // recorded contacts per body and substep (adjoint)
constexpr int JB_THREADS = 128;            // k_joint_blocks: one thread per small component
constexpr uint32_t JB_MAX_JOINTS = 64;     // larger components take the coloured sweep
constexpr uint32_t JB_JOINTS = 512;        // joints staged in shared memory per block
constexpr uint32_t JB_BODIES = 640;        // bodies staged per block (<= JB_JOINTS + JB_THREADS)
constexpr uint32_t JB_ITERS = 4;           // iterations whose rotation terms a block keeps
constexpr uint32_t JL_STATIC_A = 1u << 15; // jnt_local flags: body a / b is static
constexpr uint32_t JL_STATIC_B = 1u << 31;

}  // namespace blobs
