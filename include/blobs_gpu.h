/*
 * blobs_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the blobs
 * per-step simulation path (darthdeus/blobs 0.2.1, blobs/src/physics.rs).
 *
 * This is the thin FFI layer that a host keeping the reference's `Physics`
 * API (rigid-body / collider / spring / joint arenas, builders, handles)
 * binds to: the host hands its arenas over as structure-of-arrays in arena
 * iteration order, and `Physics::step(dt)` becomes `blobs_world_step`.
 * The C++ mirror of that host API is include/blobs_physics.hpp.
 *
 * Conventions
 *   - Every entry point returns an int status (blobs_status).  They replace
 *     the reference's panics: e.g. physics.rs:142 `expect` -> INVALID_HANDLE,
 *     physics.rs:293 / :471-474 `assert!` -> NAN.
 *   - Ownership: the world owns its device memory; all input arrays are host
 *     memory, copied during the call; the caller keeps ownership.
 *   - Threading: one world is driven by one host thread at a time (the
 *     reference Physics is !Send: physics.rs:4 holds an Rc).  Each world owns
 *     one CUDA stream; calls are asynchronous unless documented otherwise,
 *     and device-side failures are reported by the next synchronising call
 *     (a read, blobs_world_sync).
 *   - Arena order: bodies, colliders, springs and joints are given in the
 *     order the reference iterates its thunderdome arenas (ascending slot).
 *     That order is semantic: it fixes the contact pair sequence
 *     (physics.rs:244-249), the spring order (:406-408), the joint order
 *     (:426) and which body sees the `old_dt` ratio first (:338-339).
 *   - There is no CPU fallback: without a usable CUDA device the calls that
 *     need one return BLOBS_ERR_NO_DEVICE.
 */
#ifndef BLOBS_GPU_H
#define BLOBS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BLOBS_ABI_VERSION 1

typedef enum blobs_status {
  BLOBS_OK = 0,
  BLOBS_ERR_INVALID_HANDLE = 1,   /* unknown world / handle (physics.rs:142 expect) */
  BLOBS_ERR_INVALID_ARGUMENT = 2, /* bad sizes, indices, NULL where required */
  BLOBS_ERR_OVERFLOW = 3,         /* a caller-provided capacity was too small */
  BLOBS_ERR_NAN = 4,              /* NaN contact normal / non-finite rotation (physics.rs:293,471-474) */
  BLOBS_ERR_CUDA = 5,             /* a CUDA runtime call failed */
  BLOBS_ERR_TIMEOUT = 6,          /* a bounded device-side wait gave up (reserved: no kernel waits on another) */
  BLOBS_ERR_NO_DEVICE = 7,        /* no usable CUDA device */
  BLOBS_ERR_OUT_OF_MEMORY = 8,    /* device allocation failed */
  BLOBS_ERR_STATE = 9             /* call not valid in the world's current state */
} blobs_status;

/* Body types, RigidBodyType (blobs/src/rigid_body.rs:219-242).  Only Static
 * changes the step: kinematic bodies integrate like dynamic ones, exactly as
 * in the reference (which only ever tests is_static). */
enum { BLOBS_DYNAMIC = 0, BLOBS_STATIC = 1, BLOBS_KINEMATIC_POSITION = 2, BLOBS_KINEMATIC_VELOCITY = 3 };

typedef struct blobs_world blobs_world;

/* Physics knobs (physics.rs:6-27) plus the broadphase cell size. */
typedef struct blobs_config {
  float gravity[2];            /* Physics.gravity */
  uint32_t substeps;           /* physics.rs:46, default 8 */
  uint32_t joint_iterations;   /* physics.rs:47, default 4 */
  uint32_t collisions_enabled; /* physics.rs:27,62, default 1 */
  float cell_size;             /* broadphase cell edge; 0 = 2 * max collider radius * (1 + 1/64) */
  int32_t device;              /* CUDA device ordinal, default 0 */
} blobs_config;

/*
 * A whole scene in arena order.  `n_worlds` independent worlds may be packed
 * back to back (batched mode): world w owns bodies
 * [world_body_offsets[w], world_body_offsets[w+1]) and likewise colliders,
 * springs and joints; cross-world references are rejected.  With n_worlds <= 1
 * the offset arrays may be NULL.  NULL optional arrays take the defaults in
 * brackets, which are the RigidBodyBuilder / ColliderBuilder defaults
 * (rigid_body.rs:303-318, collider.rs:212-224).
 */
typedef struct blobs_scene {
  uint32_t n_worlds;
  const uint32_t* world_body_offsets;     /* n_worlds + 1 */
  const uint32_t* world_collider_offsets; /* n_worlds + 1 */
  const uint32_t* world_spring_offsets;   /* n_worlds + 1 */
  const uint32_t* world_joint_offsets;    /* n_worlds + 1 */
  const float* world_box;                 /* 4 per world (lo.x, lo.y, hi.x, hi.y) or NULL: wall extension */

  /* RigidBody fields (rigid_body.rs:42-74) */
  uint32_t n_bodies;
  const float* pos;          /* 2n  position */
  const float* pos_old;      /* 2n  position_old [= pos] */
  const float* acc;          /* 2n  acceleration [0] */
  const float* vel;          /* 2n  calculated_velocity [0] */
  const float* vreq;         /* 2n  velocity_request value */
  const uint8_t* vreq_set;   /* n   velocity_request is Some [0] */
  const uint8_t* body_type;  /* n   [DYNAMIC] */
  const float* rotation;     /* n   [0] */
  const float* angvel;       /* n   angular_velocity [0] */
  const float* torque;       /* n   [0] */
  const float* gravity_mod;  /* n   [1] */
  const float* mass;         /* n   calculated_mass: required (see blobs_body_mass_inertia) */
  const float* inertia;      /* n   required */

  /* Collider fields (collider.rs:3-20); spheres only, offset = translation */
  uint32_t n_colliders;
  const uint32_t* col_parent;  /* c   dense body index (required) */
  const float* col_offset;     /* 2c  offset.translation [0] */
  const float* col_radius;     /* c   required */
  const uint8_t* col_sensor;   /* c   flags.is_sensor [0] */
  const uint32_t* col_memb;    /* c   collision_groups.memberships [ALL] */
  const uint32_t* col_filt;    /* c   collision_groups.filter [ALL] */
  const float* col_snap;       /* 2c  absolute_transform.translation [transform(body) * offset] */

  /* Spring (springs.rs:16-22), arena order */
  uint32_t n_springs;
  const uint32_t* spr_a;
  const uint32_t* spr_b;
  const float* spr_rest;
  const float* spr_k;
  const float* spr_c;

  /* FixedJoint (joints.rs:7-19), arena order */
  uint32_t n_joints;
  const uint32_t* jnt_a;
  const uint32_t* jnt_b;
  const float* jnt_anchor_a;  /* 2j */
  const float* jnt_anchor_b;  /* 2j */
  const float* jnt_distance;  /* j */
  const float* jnt_target;    /* j  target_angle */

  /* Circle constraints (lib.rs:189-193), applied to every world */
  uint32_t n_circles;
  const float* circles;  /* 3 per circle: x, y, radius */
} blobs_scene;

/* ---- configuration / lifetime --------------------------------------------- */

/* Physics::new defaults (physics.rs:37-69): gravity (0,0), 8 substeps,
 * 4 joint iterations, collisions enabled, automatic cell size, device 0. */
void blobs_config_default(blobs_config* cfg);
const char* blobs_status_string(int status);
int blobs_abi_version(void);

/* Physics::new (physics.rs:37-69). */
int blobs_world_create(const blobs_config* cfg, blobs_world** out);
/* Drop. Frees all device memory of the world. */
int blobs_world_destroy(blobs_world* w);
/* Replace the physics knobs (gravity, substeps, ...) between steps. */
int blobs_world_set_config(blobs_world* w, const blobs_config* cfg);

/* Upload a scene, replacing the previous one (Physics::reset, physics.rs:71-76,
 * followed by the insert_* calls).  The world's `old_dt` is set to `old_dt`
 * (1.0 for a fresh Physics, physics.rs:67). */
int blobs_world_load(blobs_world* w, const blobs_scene* scene, float old_dt);

/* ---- the step -------------------------------------------------------------- */

/* Physics::step (physics.rs:78-82): `substeps` substeps of gravity, springs,
 * contacts, fixed joints, Verlet integration and constraints on every world. */
int blobs_world_step(blobs_world* w, double delta);
/* `n_steps` calls of step(delta) issued as one CUDA-graph launch. */
int blobs_world_rollout(blobs_world* w, double delta, uint32_t n_steps);
/* Physics::fixed_step (physics.rs:84-99): accumulator with delta = 1/60 and at
 * most 3 integrate calls per frame. */
int blobs_world_fixed_step(blobs_world* w, double frame_time);
/* Wait for the world's stream; returns the first device-side error, if any. */
int blobs_world_sync(blobs_world* w);

/* Run the world's work on the caller's CUDA stream (a cudaStream_t) instead of
 * its own; NULL returns to the world's own stream.  Lets a host order the
 * step with its own copies and kernels. */
int blobs_world_set_stream(blobs_world* w, void* stream);

/* ---- host writes between steps ----------------------------------------------- */

/* Overwrite body state in arena order, as a host mutating rbd.position /
 * position_old / calculated_velocity / rotation / angular_velocity through
 * Physics::get_mut_rbd (physics.rs:109-111) would.  Collider snapshots are not
 * touched, exactly like the reference (they refresh in update_objects).  Any
 * pointer may be NULL; asynchronous on the world's stream. */
int blobs_world_write_bodies(blobs_world* w, const float* pos, const float* pos_old, const float* vel,
                             const float* rotation, const float* angvel);

/* ---- snapshot / restore (no reference counterpart) -------------------------- */

/* Copy the world's whole device state -- every array of the loaded scene
 * (positions, previous positions, velocities, rotations, collider snapshots,
 * pending velocity requests, cell tables, contact counters) -- and its step
 * bookkeeping (old_dt, time, fixed-step accumulator) into a snapshot the
 * world holds (one per world, device memory the size of the scene), and
 * restore it: stepping after a restore repeats the steps taken after the
 * snapshot bit for bit.  Device-to-device and asynchronous on the world's
 * stream.  Loading a scene drops the snapshot; restoring drops a recorded
 * rollout; the collision-event buffer is not part of the state. */
int blobs_world_snapshot(blobs_world* w);
int blobs_world_restore(blobs_world* w);

/* ---- per-phase device timing (profiling aid; no reference counterpart) ------ */

/* Number of kernels this world has issued (eagerly or as nodes of a launched
 * graph) since it was created. */
int blobs_world_kernel_launches(blobs_world* w, uint64_t* count);

/* enabled = 1: CUDA events are recorded around each kernel phase of every
 * substep (inside the step graphs); 2: around the contact phase only (its
 * kernel timed without event nodes between the other kernels); 0: off. */
int blobs_world_set_timing(blobs_world* w, int enabled);
/* Device milliseconds and launch counts per phase since the previous call:
 * [0] cell scan, [1] scatter + forces, [2] contacts (+ fused integration),
 * [3] fixed joints, [4] integration.  n_phases >= 5.  Synchronising. */
int blobs_world_phase_times(blobs_world* w, double* ms, uint64_t* launches, uint32_t n_phases);

/* ---- reads (synchronising) ------------------------------------------------- */

/* Body state in arena order: position, position_old, calculated_velocity,
 * rotation, angular_velocity.  Any pointer may be NULL. */
int blobs_world_read_bodies(blobs_world* w, float* pos, float* pos_old, float* vel, float* rotation,
                            float* angvel);
/* Collider absolute translations (Physics::col_position, physics.rs:155-157). */
int blobs_world_read_snapshots(blobs_world* w, float* xy);
/* Contacts counted by the contact pass: total since load and in the last
 * substep (the reference's perf counter "collisions", physics.rs:316). */
int blobs_world_contact_count(blobs_world* w, uint64_t* total, uint64_t* last_substep);
/* Contacts resolved with the coincident-centre push-out branch
 * (physics.rs:272-286) since load. */
int blobs_world_pushout_count(blobs_world* w, uint64_t* total);
/* No counterpart in the reference (a cost diagnostic): bodies of the
 * single-sphere path whose 3x3 cells held more than 64 candidates, or which
 * had more near candidates than the step kernel takes (32 in the plain step
 * of a uniform world, 12 otherwise), and whose contacts were therefore
 * resolved by a warp of their own -- since load and in the last substep. */
int blobs_world_deferred_count(blobs_world* w, uint64_t* total, uint64_t* last_substep);
/* The broadphase output for the current collider snapshots: every collider
 * pair (hi, lo), hi > lo in arena order, whose cells are 3x3 neighbours in
 * its world's grid (contacts_only = 0), or only the pairs the contact pass
 * resolves (contacts_only = 1: different parents, InteractionGroups::test,
 * distance < ra + rb -- the pair set of brute_force_collisions,
 * physics.rs:248-269).  Unordered; `pairs` holds 2 * cap entries.  Returns
 * BLOBS_ERR_OVERFLOW with *n_pairs = the full count when cap is too small. */
int blobs_world_emit_pairs(blobs_world* w, int contacts_only, uint32_t* pairs, uint64_t cap, uint64_t* n_pairs);
/* The toroidal cell grid of world `world`: cell edge, its f32 reciprocal,
 * the origin (2 floats) and log2 of the width and height in cells
 * (cell (ix, iy) = floor((v - origin) * inv_cell_size) in f32, wrapped mod
 * 2^log2). */
int blobs_world_grid(blobs_world* w, uint32_t world, float* cell_size, float* inv_cell_size, float* origin,
                     uint32_t* log2_width, uint32_t* log2_height);
/* Physics.time and the accumulator of fixed_step. */
int blobs_world_time(blobs_world* w, double* time, double* accumulator);
/* The joint processing order of the GPU schedule: the joints of components
 * of at most 64 joints, component by component, each in arena order (which
 * gives every body the reference's own sequence of updates), then the joints
 * of larger components by graph colour, then arena index.  Sweeping the
 * joints in this order, joint_iterations times, reproduces the GPU's result.
 * `order` holds n_joints entries; `n_colours` counts the large components'
 * colours (0 when every component is small). */
int blobs_world_joint_order(blobs_world* w, uint32_t* order, uint32_t* n_colours);
/* The same schedule computed on the host for a joint list alone (no device):
 * `order` (n_joints) as above; block k of the small components sweeps
 * order[block_joint_start[k] .. block_joint_start[k+1]) (n_blocks + 1 entries,
 * at most n_joints + 1); colour k of the large components is
 * order[colour_start[k] .. colour_start[k+1]) (n_colours + 1 entries, at most
 * n_joints + 1).  Output pointers may be NULL. */
int blobs_joint_schedule(uint32_t n_bodies, uint32_t n_joints, const uint32_t* jnt_a, const uint32_t* jnt_b,
                         uint32_t* order, uint32_t* block_joint_start, uint32_t* n_blocks, uint32_t* colour_start,
                         uint32_t* n_colours);

/* ---- differentiable rollout (no counterpart in the reference) ---------------- */

/* `n_steps` calls of step(delta) on a single-sphere world (every body one
 * collider at offset zero, default groups, no sensor, no joints, no circle
 * constraint; springs, walls, static bodies and batched worlds allowed),
 * keeping the arena-order state every `checkpoint_every` steps for
 * blobs_world_backward.  The velocity requests pending at the start (the
 * RigidBodyBuilder::velocity_request of a fresh scene, rigid_body.rs:346-349)
 * and the spring stiffnesses are the differentiable parameters. */
int blobs_world_rollout_record(blobs_world* w, double delta, uint32_t n_steps, uint32_t checkpoint_every);
/* Reverse pass of the last recorded rollout: given dL/d(final position)
 * (2 n_bodies floats, host), writes dL/d(velocity request) (2 n_bodies,
 * host, may be NULL) and dL/d(spring stiffness) (n_springs, host, may be
 * NULL).  Each checkpoint segment is recomputed (bit-identical to the
 * forward pass) with its contacts recorded, then reversed substep by
 * substep.  Contacts resolved by the push-out branch (coincident centres,
 * physics.rs:272-286) are not differentiated.  The world is left in the
 * rollout's final state.  A reload, a change of the substep count or of the
 * event mode drops the recording (then BLOBS_ERR_STATE).  Every sum runs
 * in a fixed order: the gradients are deterministic.  Allocates its scratch
 * per call: 92 B per body per substep of one checkpoint segment (the state
 * after the substep and up to 16 recorded contacts); a body with more than
 * 16 contacts in one substep gives BLOBS_ERR_OVERFLOW.  The derivative of
 * long contact-rich rollouts can exceed the f32 range; such gradients come
 * back as +-inf or NaN with BLOBS_OK.  Synchronising. */
int blobs_world_backward(blobs_world* w, const float* dl_dpos, float* dl_dvreq, float* dl_dk);

/* Autotuner (no counterpart in the reference): loads `scene` with each of a
 * few broadphase cell edges (1, 1.125, 1.25, 1.5 and 1.75 times the smallest
 * exact edge, 2 x largest radius x (1 + 1/64)), times `trial_steps` steps
 * of `delta` from the scene's initial state on the world's stream, keeps the
 * fastest (*cell_scale, may be NULL) and reloads the scene with it.  Every
 * such edge gives the same contacts in the same order: the results do not
 * depend on the choice.  A later blobs_world_load keeps the chosen scale.
 * Synchronising. */
int blobs_world_autotune(blobs_world* w, const blobs_scene* scene, float old_dt, double delta, uint32_t trial_steps,
                         float* cell_scale);

/* ---- collision events -------------------------------------------------------- */

/* Replaces the CollisionEvent channel (lib.rs:146-153): Physics::new's
 * std::sync::mpsc channel (physics.rs:37) and the send of one event per
 * resolved pair in brute_force_collisions (physics.rs:304-311).  Off by
 * default (events cost device bandwidth); enabled, every contact pass
 * appends (collider a, collider b, impact_vel_a, impact_vel_b) for each
 * pair in contact -- a > b in arena order, sensors included, the impact
 * velocities being the parents' calculated_velocity at the start of the
 * pass -- into a device buffer of `capacity` events.  Enabling or disabling
 * discards undrained events; a reload (blobs_world_load) starts a new
 * stream.  Batched worlds share one stream with scene-global collider
 * indices.  Not synchronising. */
int blobs_world_set_events(blobs_world* w, int enabled, uint32_t capacity);
/* collision_recv.try_iter(): moves the events produced since the last drain
 * to the host in the reference's order (substep by substep; outer collider
 * ascending, then inner collider ascending) and writes up to `cap` of them
 * (impact velocities as 2 floats each; either velocity array may be NULL).
 * *n_written = events written, *n_left (may be NULL) = events kept for the
 * next call.  If the device buffer overflowed since the last drain the
 * whole batch is dropped (it is not a prefix of the reference's order):
 * returns BLOBS_ERR_OVERFLOW with *n_left = events produced, so the caller
 * can enlarge the capacity.  BLOBS_ERR_STATE when events are off.
 * Synchronising. */
int blobs_world_drain_events(blobs_world* w, uint32_t* col_a, uint32_t* col_b, float* impact_vel_a,
                             float* impact_vel_b, uint64_t cap, uint64_t* n_written, uint64_t* n_left);

/* ---- spatial hash queries ---------------------------------------------------- */

/* SpatialHash (blobs/src/spatial.rs:31-195) on a device: a set of points
 * (id, position, radius) bucketed by the reference's integer cell
 * ((x / cell_size).floor() as i32, same for y; spatial.rs:57-62), and
 * SpatialHash::query (spatial.rs:155-195) for many query points at once. */
typedef struct blobs_spatial_hash blobs_spatial_hash;
/* SpatialHash::new (spatial.rs:45-56). */
int blobs_spatial_hash_create(float cell_size, int32_t device, blobs_spatial_hash** out);
int blobs_spatial_hash_destroy(blobs_spatial_hash* h);
/* Replaces the point set, as insert_with_id (spatial.rs:71-84) of every point
 * into an empty hash: n points, ids unique (duplicate ids give unspecified
 * results), xy 2n floats, radius n floats; host memory, copied.
 * Synchronising. */
int blobs_spatial_hash_set_points(blobs_spatial_hash* h, uint64_t n, const uint64_t* ids, const float* xy,
                                  const float* radius);
/* SpatialHash::query for nq query points (qxy 2nq floats, qradius nq):
 * every point of the 3x3 cells around the query point's cell with
 * |p - q|^2 <= (query_radius + radius)^2.  offsets (nq + 1, host) delimit
 * each query's ids in `ids` (host, ascending per query; the reference's order
 * is its HashMap's, unspecified).  *total = number of results; if it exceeds
 * `cap` nothing is written to `ids` and BLOBS_ERR_OVERFLOW is returned with
 * the offsets filled (call again with cap >= *total).  Synchronising. */
int blobs_spatial_hash_query(blobs_spatial_hash* h, uint64_t nq, const float* qxy, const float* qradius,
                             uint64_t* offsets, uint64_t* ids, uint64_t cap, uint64_t* total);

/* ---- contact pairs without any allocation ------------------------------------ */

/* No counterpart in the reference.  The contact pair set of
 * blobs_world_emit_pairs(contacts_only = 1) -- pairs (hi, lo), hi > lo, with
 * different parents, passing InteractionGroups::test and closer than the sum
 * of their radii -- for `n` colliders already in device memory, computed
 * without a world and without allocating: for hosts that must not call
 * cudaMalloc / cudaFree while they run (those calls synchronise the whole
 * device, which a frame loop cannot absorb) or whose device memory belongs to
 * their own budgeted allocator.  All scratch lives in one static device array
 * of this library sized for at most blobs_noalloc_max_colliders() (65,536)
 * colliders; every GPU that loads the library holds it (about 2.3 MB) until
 * the process exits.  Larger n is rejected with BLOBS_ERR_INVALID_ARGUMENT.
 *   snap: 2n floats (device), radius: n floats (device); parent / memb / filt:
 *   n uint32 (device) or NULL (all different / all groups);
 *   pairs: 2 * cap uint32 (device); count: one device counter that receives
 *   the full number of pairs (pairs past `cap` are counted, not written).
 * Any finite coordinates are exact (no pair is lost far from the origin); a
 * non-finite snapshot or a NaN radius gives no pair, a +inf radius a pair
 * with every collider the filters allow -- as in the world path.
 * Asynchronous on `stream` (a cudaStream_t, NULL = the legacy default).  The
 * first call on a device looks up the device address of the scratch array
 * (once, with that device current); make that first call before any stream
 * capture.  Every call reuses the same scratch array, so calls whose work
 * overlaps on the GPU race: issue them on one stream, or wait for the
 * previous one. */
int blobs_contact_pairs_noalloc(uint32_t n, const float* snap, const float* radius, const uint32_t* parent,
                                const uint32_t* memb, const uint32_t* filt, uint32_t* pairs, uint64_t cap,
                                unsigned long long* count, void* stream);
/* The largest collider count blobs_contact_pairs_noalloc accepts. */
uint32_t blobs_noalloc_max_colliders(void);

/* ---- host-side helpers (no device needed) ---------------------------------- */

/* RigidBody::update_mass_and_inertia (rigid_body.rs:96-128) for every body,
 * including the reference's double registration of each collider handle
 * (collider.rs:180 and physics.rs:144): mass = sum over handles of
 * (mass_override or 2r) counted twice, sensors skipped, 0 -> 1.
 * col_mass_override: NaN means None; the array may be NULL. */
int blobs_body_mass_inertia(uint32_t n_bodies, uint32_t n_colliders, const uint32_t* col_parent,
                            const float* col_offset, const float* col_radius, const float* col_mass_override,
                            const uint8_t* col_sensor, float* mass_out, float* inertia_out);

#ifdef __cplusplus
}
#endif

#endif /* BLOBS_GPU_H */
