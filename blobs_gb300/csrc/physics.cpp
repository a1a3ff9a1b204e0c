// physics.cpp -- the C++ host mirror of the reference Physics API
// (include/blobs_physics.hpp) on top of the C ABI (include/blobs_gpu.h).
#include "blobs_physics.hpp"

#include <algorithm>
#include <cstring>

namespace blobs {

namespace {
void check(int st, const char* what) {
  if (st != BLOBS_OK) throw Error(st, what);
}
}  // namespace

// rigid_body.rs:96-128
void RigidBody::update_mass_and_inertia(const Arena<Collider>& col_set) {
  calculated_mass = 0.0f;
  inertia = 0.0f;
  Vec2 weighted;
  for (const ColliderHandle& h : colliders) {
    const Collider* c = col_set.get(h.idx);
    if (!c) continue;  // the reference logs "Collider not found" and skips it
    if (c->is_sensor) continue;
    const float m = c->mass();
    calculated_mass += m;
    inertia += c->inertia();
    weighted += c->offset * m;
  }
  if (calculated_mass == 0.0f) calculated_mass = 1.0f;
  if (inertia == 0.0f) inertia = 1.0f;
  center_of_mass = weighted / calculated_mass;
}

Physics::Physics(Vec2 g, bool use_sh, int device) : gravity(g), use_spatial_hash(use_sh), device_(device) {}

Physics::~Physics() {
  if (world_) blobs_world_destroy(world_);
}

void Physics::reset() {
  pull();
  rbd_set_.clear();
  col_set_.clear();
  joints_.clear();
  springs_.clear();
  host_dirty_ = true;
}

std::optional<RigidBodyData> Physics::get_rbd_data(RigidBodyHandle h) {
  const RigidBody* b = get_rbd(h);
  if (!b) return std::nullopt;
  return b->data();
}

const RigidBody* Physics::get_rbd(RigidBodyHandle h) {
  pull();
  return rbd_set_.get(h.idx);
}

RigidBody* Physics::get_mut_rbd(RigidBodyHandle h) {
  pull();
  RigidBody* b = rbd_set_.get(h.idx);
  if (b) host_dirty_ = true;  // the caller may change anything through the reference
  return b;
}

const Collider* Physics::get_col(ColliderHandle h) {
  pull();
  return col_set_.get(h.idx);
}

RigidBodyHandle Physics::insert_rbd(RigidBody rbd) {
  pull();
  host_dirty_ = true;
  return RigidBodyHandle{rbd_set_.insert(std::move(rbd))};
}

ColliderHandle Physics::insert_collider_with_parent(Collider c, RigidBodyHandle parent) {
  pull();
  c.parent = parent;
  ColliderHandle ch{col_set_.insert(std::move(c))};
  RigidBody* b = rbd_set_.get(parent.idx);
  if (!b) {
    // collider.rs:179 skips the push, then physics.rs:139-142 panics
    throw Error(BLOBS_ERR_INVALID_HANDLE, "parent rigid body must exist when inserting collider");
  }
  b->colliders.push_back(ch);  // collider.rs:180
  b->colliders.push_back(ch);  // physics.rs:144 (the handle is registered twice)
  b->update_mass_and_inertia(col_set_);
  host_dirty_ = true;
  return ch;
}

std::optional<Vec2> Physics::rbd_position(RigidBodyHandle h) {
  const RigidBody* b = get_rbd(h);
  if (!b) return std::nullopt;
  return b->position;
}

std::optional<Vec2> Physics::col_position(ColliderHandle h) {
  const Collider* c = get_col(h);
  if (!c) return std::nullopt;
  return c->absolute_translation;
}

// ColliderSet::remove (collider.rs:134-164)
void Physics::remove_col(ColliderHandle h) {
  pull();
  const Collider* c = col_set_.get(h.idx);
  if (c && c->parent) {
    const RigidBodyHandle parent = *c->parent;
    RigidBody* b = rbd_set_.get(parent.idx);
    bool remove_body = false;
    if (b) {
      std::vector<ColliderHandle> keep;
      for (const ColliderHandle& x : b->colliders)
        if (!(x == h)) keep.push_back(x);
      b->colliders.swap(keep);
      b->update_mass_and_inertia(col_set_);
      remove_body = b->colliders.empty();
    }
    if (remove_body) rbd_set_.remove(parent.idx);
  }
  col_set_.remove(h.idx);
  host_dirty_ = true;
}

// physics.rs:163-172
void Physics::remove_rbd(RigidBodyHandle h) {
  pull();
  if (const RigidBody* b = rbd_set_.get(h.idx)) {
    const std::vector<ColliderHandle> cols = b->colliders;
    for (const ColliderHandle& c : cols) col_set_.remove(c.idx);
  }
  rbd_set_.remove(h.idx);
  host_dirty_ = true;
}

// physics.rs:174-182
void Physics::update_rigid_body_position(uint64_t id, Vec2 offset) {
  pull();
  if (RigidBody* b = rbd_set_.get(Index::from_bits(id))) {
    b->position += offset;
    host_dirty_ = true;
  }
}

// physics.rs:184-207
JointHandle Physics::create_fixed_joint(RigidBodyHandle a, RigidBodyHandle b, Vec2 anchor_a, Vec2 anchor_b) {
  pull();
  const RigidBody* ra = rbd_set_.get(a.idx);
  const RigidBody* rb = rbd_set_.get(b.idx);
  if (!ra || !rb || a == b) throw Error(BLOBS_ERR_INVALID_HANDLE, "create_fixed_joint");
  const float distance = (ra->position + anchor_a - rb->position - anchor_b).length();
  return create_fixed_joint_with_distance(a, b, anchor_a, anchor_b, distance);
}

// physics.rs:209-239
JointHandle Physics::create_fixed_joint_with_distance(RigidBodyHandle a, RigidBodyHandle b, Vec2 anchor_a,
                                                      Vec2 anchor_b, float distance) {
  pull();
  RigidBody* ra = rbd_set_.get(a.idx);
  RigidBody* rb = rbd_set_.get(b.idx);
  if (!ra || !rb || a == b) throw Error(BLOBS_ERR_INVALID_HANDLE, "create_fixed_joint_with_distance");
  FixedJoint j{a, b, anchor_a, anchor_b, distance, rb->rotation - ra->rotation};
  JointHandle jh{joints_.insert(j)};
  ra->connected_joints.push_back(jh);
  rb->connected_joints.push_back(jh);
  host_dirty_ = true;
  return jh;
}

SpringHandle Physics::insert_spring(Spring s) {
  pull();
  host_dirty_ = true;
  return SpringHandle{springs_.insert(s)};
}

void Physics::remove_spring(SpringHandle h) {
  pull();
  springs_.remove(h.idx);
  host_dirty_ = true;
}

uint64_t Physics::contact_count() {
  if (!world_ || host_dirty_) return 0;
  uint64_t total = 0;
  check(blobs_world_contact_count(world_, &total, nullptr), "blobs_world_contact_count");
  return total;
}

void Physics::push() {
  blobs_config cfg;
  blobs_config_default(&cfg);
  cfg.gravity[0] = gravity.x;
  cfg.gravity[1] = gravity.y;
  cfg.substeps = substeps;
  cfg.joint_iterations = joint_iterations;
  cfg.collisions_enabled = collisions_enabled ? 1u : 0u;
  cfg.device = device_;
  if (!world_) {
    check(blobs_world_create(&cfg, &world_), "blobs_world_create");
  } else {
    check(blobs_world_set_config(world_, &cfg), "blobs_world_set_config");
  }
  if (!host_dirty_) return;

  // dense arrays in arena iteration order
  body_slots_.clear();
  col_slots_.clear();
  std::vector<int64_t> body_dense;
  std::vector<float> pos, pos_old, acc, vel, vreq, rot, av, tq, gmod, mass, inertia;
  std::vector<uint8_t> vset, type;
  rbd_set_.for_each([&](Index i, const RigidBody& b) {
    if (body_dense.size() <= i.slot) body_dense.resize(i.slot + 1, -1);
    body_dense[i.slot] = (int64_t)body_slots_.size();
    body_slots_.push_back(i);
    pos.insert(pos.end(), {b.position.x, b.position.y});
    pos_old.insert(pos_old.end(), {b.position_old.x, b.position_old.y});
    acc.insert(acc.end(), {b.acceleration.x, b.acceleration.y});
    vel.insert(vel.end(), {b.calculated_velocity.x, b.calculated_velocity.y});
    const Vec2 vr = b.velocity_request ? *b.velocity_request : Vec2();
    vreq.insert(vreq.end(), {vr.x, vr.y});
    vset.push_back(b.velocity_request ? 1 : 0);
    type.push_back((uint8_t)b.body_type);
    rot.push_back(b.rotation);
    av.push_back(b.angular_velocity);
    tq.push_back(b.torque);
    gmod.push_back(b.gravity_mod);
    mass.push_back(b.calculated_mass);
    inertia.push_back(b.inertia);
  });
  auto dense_body = [&](RigidBodyHandle h) -> int64_t {
    if (!rbd_set_.contains(h.idx) || h.idx.slot >= body_dense.size()) return -1;
    return body_dense[h.idx.slot];
  };
  std::vector<uint32_t> cparent, memb, filt;
  std::vector<float> coff, crad, csnap;
  std::vector<uint8_t> csens;
  col_set_.for_each([&](Index i, const Collider& c) {
    if (!c.parent) return;  // physics.rs:252-253: parentless colliders never collide
    const int64_t p = dense_body(*c.parent);
    if (p < 0) return;
    col_slots_.push_back(i);
    cparent.push_back((uint32_t)p);
    coff.insert(coff.end(), {c.offset.x, c.offset.y});
    crad.push_back(c.radius);
    csens.push_back(c.is_sensor ? 1 : 0);
    memb.push_back(c.collision_groups.memberships);
    filt.push_back(c.collision_groups.filter);
    csnap.insert(csnap.end(), {c.absolute_translation.x, c.absolute_translation.y});
  });
  std::vector<uint32_t> sa, sb;
  std::vector<float> srest, sk, sc;
  springs_.for_each([&](Index, const Spring& s) {
    const int64_t a = dense_body(s.rigid_body_a), b = dense_body(s.rigid_body_b);
    if (a < 0 || b < 0) throw Error(BLOBS_ERR_INVALID_HANDLE, "spring refers to a removed rigid body");
    sa.push_back((uint32_t)a);
    sb.push_back((uint32_t)b);
    srest.push_back(s.rest_length);
    sk.push_back(s.stiffness);
    sc.push_back(s.damping);
  });
  std::vector<uint32_t> ja, jb;
  std::vector<float> jaa, jab, jd, jt;
  joints_.for_each([&](Index, const FixedJoint& j) {
    const int64_t a = dense_body(j.rigid_body_a), b = dense_body(j.rigid_body_b);
    if (a < 0 || b < 0) throw Error(BLOBS_ERR_INVALID_HANDLE, "joint refers to a removed rigid body");
    ja.push_back((uint32_t)a);
    jb.push_back((uint32_t)b);
    jaa.insert(jaa.end(), {j.anchor_a.x, j.anchor_a.y});
    jab.insert(jab.end(), {j.anchor_b.x, j.anchor_b.y});
    jd.push_back(j.distance);
    jt.push_back(j.target_angle);
  });
  std::vector<float> circles;
  for (const Constraint& k : constraints) circles.insert(circles.end(), {k.position.x, k.position.y, k.radius});
  float box[4];
  if (walls) {
    box[0] = walls->first.x;
    box[1] = walls->first.y;
    box[2] = walls->second.x;
    box[3] = walls->second.y;
  }

  blobs_scene s;
  std::memset(&s, 0, sizeof(s));
  s.n_worlds = 1;
  s.world_box = walls ? box : nullptr;
  s.n_bodies = (uint32_t)body_slots_.size();
  s.pos = pos.data();
  s.pos_old = pos_old.data();
  s.acc = acc.data();
  s.vel = vel.data();
  s.vreq = vreq.data();
  s.vreq_set = vset.data();
  s.body_type = type.data();
  s.rotation = rot.data();
  s.angvel = av.data();
  s.torque = tq.data();
  s.gravity_mod = gmod.data();
  s.mass = mass.data();
  s.inertia = inertia.data();
  s.n_colliders = (uint32_t)col_slots_.size();
  s.col_parent = cparent.data();
  s.col_offset = coff.data();
  s.col_radius = crad.data();
  s.col_sensor = csens.data();
  s.col_memb = memb.data();
  s.col_filt = filt.data();
  s.col_snap = csnap.data();
  s.n_springs = (uint32_t)sa.size();
  s.spr_a = sa.data();
  s.spr_b = sb.data();
  s.spr_rest = srest.data();
  s.spr_k = sk.data();
  s.spr_c = sc.data();
  s.n_joints = (uint32_t)ja.size();
  s.jnt_a = ja.data();
  s.jnt_b = jb.data();
  s.jnt_anchor_a = jaa.data();
  s.jnt_anchor_b = jab.data();
  s.jnt_distance = jd.data();
  s.jnt_target = jt.data();
  s.n_circles = (uint32_t)constraints.size();
  s.circles = circles.data();
  check(blobs_world_load(world_, &s, old_dt), "blobs_world_load");
  host_dirty_ = false;
}

void Physics::pull() {
  if (!device_newer_ || !world_) return;
  const size_t n = body_slots_.size(), c = col_slots_.size();
  std::vector<float> pos(2 * n), pos_old(2 * n), vel(2 * n), rot(n), av(n), snap(2 * c);
  check(blobs_world_read_bodies(world_, pos.data(), pos_old.data(), vel.data(), rot.data(), av.data()),
        "blobs_world_read_bodies");
  if (c) check(blobs_world_read_snapshots(world_, snap.data()), "blobs_world_read_snapshots");
  for (size_t i = 0; i < n; ++i) {
    RigidBody* b = rbd_set_.get(body_slots_[i]);
    b->position = Vec2(pos[2 * i], pos[2 * i + 1]);
    b->position_old = Vec2(pos_old[2 * i], pos_old[2 * i + 1]);
    b->calculated_velocity = Vec2(vel[2 * i], vel[2 * i + 1]);
    b->rotation = rot[i];
    b->angular_velocity = av[i];
    // consumed by update_objects (physics.rs:327-355)
    b->acceleration = Vec2();
    if (!b->is_static()) {
      b->velocity_request.reset();
      b->torque = 0.0f;
    }
  }
  for (size_t k = 0; k < c; ++k) col_set_.get(col_slots_[k])->absolute_translation = Vec2(snap[2 * k], snap[2 * k + 1]);
  device_newer_ = false;
}

void Physics::integrate(double delta) {
  push();
  const uint32_t want = record_collision_events
                            ? (uint32_t)std::min<uint64_t>(std::max<uint64_t>(65536, 64ull * col_slots_.size() *
                                                                                        substeps / 8),
                                                           0x7fffffffull)
                            : 0u;
  if (want > event_capacity_ || (!want && event_capacity_)) {
    check(blobs_world_set_events(world_, want ? 1 : 0, want), "blobs_world_set_events");
    event_capacity_ = want;
  }
  check(blobs_world_step(world_, delta), "blobs_world_step");
  device_newer_ = true;
  if (event_capacity_) drain_events();
  bool any_dynamic = false;
  rbd_set_.for_each([&](Index, const RigidBody& b) { any_dynamic = any_dynamic || !b.is_static(); });
  if (any_dynamic) old_dt = (float)delta / (float)substeps;  // physics.rs:339, last substep's dt
}

// Moves the device's events of the last step into events_ with handles.
void Physics::drain_events() {
  uint64_t n = 0, left = 0;
  int st = blobs_world_drain_events(world_, nullptr, nullptr, nullptr, nullptr, 0, &n, &left);
  if (st == BLOBS_ERR_OVERFLOW) {
    // a step produced more events than the buffer holds: they are lost;
    // enlarge the buffer for the next steps and report it
    event_capacity_ = (uint32_t)std::min<uint64_t>(2 * left, 0x7fffffffull);
    check(blobs_world_set_events(world_, 1, event_capacity_), "blobs_world_set_events");
  }
  check(st, "blobs_world_drain_events");
  if (!left) return;
  std::vector<uint32_t> a(left), b(left);
  std::vector<float> va(2 * left), vb(2 * left);
  check(blobs_world_drain_events(world_, a.data(), b.data(), va.data(), vb.data(), left, &n, nullptr),
        "blobs_world_drain_events");
  for (uint64_t k = 0; k < n; ++k) {
    if (a[k] >= col_slots_.size() || b[k] >= col_slots_.size())
      throw Error(BLOBS_ERR_INVALID_ARGUMENT, "collision event outside the collider arena");
    events_.push_back(CollisionEvent{ColliderHandle{col_slots_[a[k]]}, ColliderHandle{col_slots_[b[k]]},
                                     Vec2(va[2 * k], va[2 * k + 1]), Vec2(vb[2 * k], vb[2 * k + 1])});
  }
}

std::vector<CollisionEvent> Physics::collision_events() {
  std::vector<CollisionEvent> out;
  out.swap(events_);
  return out;
}

void Physics::step(double delta) {
  integrate(delta);
  time += delta;
}

void Physics::fixed_step(double frame_time) {
  accumulator += frame_time;
  const double delta = 1.0 / 60.0;
  int max_steps = 3;
  while (accumulator >= delta && max_steps > 0) {
    integrate(delta);
    accumulator -= delta;
    time += delta;
    max_steps -= 1;
  }
}

}  // namespace blobs
