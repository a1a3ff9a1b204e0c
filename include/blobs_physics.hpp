// blobs_physics.hpp -- C++ host mirror of the reference `Physics` API
// (darthdeus/blobs 0.2.1: blobs/src/physics.rs, rigid_body.rs, collider.rs,
// joints.rs, springs.rs, groups.rs, lib.rs), driving the GB300 step through
// the C ABI of blobs_gpu.h.
//
// The host keeps the arenas exactly like the reference: generational slots
// (thunderdome::Arena semantics: LIFO slot reuse, generation bumped on
// removal, iteration in ascending slot order), builders with the reference
// defaults, the doubled collider registration that doubles mass and inertia
// (collider.rs:180 + physics.rs:144).  step() uploads the arenas when the
// host changed them, runs the step on the device, and marks the host copy
// stale; the next read pulls the state back.  There is no CPU step: without
// a device, step() throws.
#pragma once

#include <cmath>
#include <cstdint>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "blobs_gpu.h"

namespace blobs {

struct Vec2 {
  float x = 0.0f, y = 0.0f;
  Vec2() = default;
  Vec2(float x_, float y_) : x(x_), y(y_) {}
  Vec2 operator+(Vec2 o) const { return {x + o.x, y + o.y}; }
  Vec2 operator-(Vec2 o) const { return {x - o.x, y - o.y}; }
  Vec2 operator-() const { return {-x, -y}; }
  Vec2 operator*(float s) const { return {x * s, y * s}; }
  Vec2 operator/(float s) const { return {x / s, y / s}; }
  Vec2& operator+=(Vec2 o) { x = x + o.x; y = y + o.y; return *this; }
  Vec2& operator-=(Vec2 o) { x = x - o.x; y = y - o.y; return *this; }
  bool operator==(Vec2 o) const { return x == o.x && y == o.y; }
  float dot(Vec2 o) const { return (x * o.x) + (y * o.y); }
  float length() const { return std::sqrt(dot(*this)); }
  static Vec2 zero() { return {0.0f, 0.0f}; }
};

/// thunderdome::Index: slot + generation; to_bits = generation << 32 | slot.
struct Index {
  uint32_t slot = 0;
  uint32_t generation = 0;
  uint64_t to_bits() const { return ((uint64_t)generation << 32) | slot; }
  static Index from_bits(uint64_t b) { return Index{(uint32_t)b, (uint32_t)(b >> 32)}; }
  bool operator==(const Index& o) const { return slot == o.slot && generation == o.generation; }
  bool operator!=(const Index& o) const { return !(*this == o); }
};

struct RigidBodyHandle { Index idx; bool operator==(const RigidBodyHandle& o) const { return idx == o.idx; } };
struct ColliderHandle { Index idx; bool operator==(const ColliderHandle& o) const { return idx == o.idx; } };
struct JointHandle { Index idx; bool operator==(const JointHandle& o) const { return idx == o.idx; } };
struct SpringHandle { Index idx; bool operator==(const SpringHandle& o) const { return idx == o.idx; } };

/// CollisionEvent (lib.rs:146-153): one per pair in contact per substep.
struct CollisionEvent {
  ColliderHandle col_handle_a;
  ColliderHandle col_handle_b;
  Vec2 impact_vel_a;
  Vec2 impact_vel_b;
};

/// Generational arena with thunderdome's observable behaviour.
template <class T> class Arena {
 public:
  Index insert(T value) {
    if (!free_.empty()) {
      uint32_t slot = free_.back();
      free_.pop_back();
      Entry& e = entries_[slot];
      e.value = std::move(value);
      e.live = true;
      ++len_;
      return Index{slot, e.generation};
    }
    entries_.push_back(Entry{std::move(value), 1u, true});
    ++len_;
    return Index{(uint32_t)(entries_.size() - 1), 1u};
  }
  std::optional<T> remove(Index i) {
    if (!contains(i)) return std::nullopt;
    Entry& e = entries_[i.slot];
    e.live = false;
    e.generation += 1;
    free_.push_back(i.slot);
    --len_;
    return std::move(e.value);
  }
  bool contains(Index i) const {
    return i.slot < entries_.size() && entries_[i.slot].live && entries_[i.slot].generation == i.generation;
  }
  T* get(Index i) { return contains(i) ? &entries_[i.slot].value : nullptr; }
  const T* get(Index i) const { return contains(i) ? &entries_[i.slot].value : nullptr; }
  size_t len() const { return len_; }
  void clear() {
    for (uint32_t s = 0; s < entries_.size(); ++s)
      if (entries_[s].live) {
        entries_[s].live = false;
        entries_[s].generation += 1;
        free_.push_back(s);
      }
    len_ = 0;
  }
  /// Live entries in ascending slot order (the reference iteration order).
  template <class F> void for_each(F&& f) {
    for (uint32_t s = 0; s < entries_.size(); ++s)
      if (entries_[s].live) f(Index{s, entries_[s].generation}, entries_[s].value);
  }
  template <class F> void for_each(F&& f) const {
    for (uint32_t s = 0; s < entries_.size(); ++s)
      if (entries_[s].live) f(Index{s, entries_[s].generation}, entries_[s].value);
  }

 private:
  struct Entry {
    T value;
    uint32_t generation;
    bool live;
  };
  std::vector<Entry> entries_;
  std::vector<uint32_t> free_;
  size_t len_ = 0;
};

enum class RigidBodyType : uint8_t { Dynamic = 0, Static = 1, KinematicPositionBased = 2, KinematicVelocityBased = 3 };

/// InteractionGroups (groups.rs:1-57).
struct InteractionGroups {
  uint32_t memberships = 0xffffffffu;
  uint32_t filter = 0xffffffffu;
  static InteractionGroups all() { return {0xffffffffu, 0xffffffffu}; }
  static InteractionGroups none() { return {0u, 0u}; }
  bool test(InteractionGroups rhs) const {
    return (memberships & rhs.filter) != 0 && (rhs.memberships & filter) != 0;
  }
};

/// RigidBodyData (rigid_body.rs:18-39).
struct RigidBodyData {
  Vec2 position, velocity;
  float angular_velocity = 0.0f;
  Vec2 center_of_mass;
  float mass = 1.0f, rotation = 0.0f;
};

class Collider;

/// RigidBody (rigid_body.rs:41-214).
struct RigidBody {
  Vec2 position, position_old, center_of_mass;
  float calculated_mass = 1.0f, gravity_mod = 1.0f, rotation = 0.0f, angular_velocity = 0.0f, torque = 0.0f,
        inertia = 1.0f;
  Vec2 scale{1.0f, 1.0f};
  Vec2 acceleration;
  std::optional<Vec2> velocity_request;
  Vec2 calculated_velocity;
  std::vector<ColliderHandle> colliders;
  std::vector<JointHandle> connected_joints;
  uint64_t user_data_lo = 0, user_data_hi = 0;
  RigidBodyType body_type = RigidBodyType::Dynamic;

  RigidBodyData data() const {
    return RigidBodyData{position, calculated_velocity, angular_velocity, center_of_mass, calculated_mass, rotation};
  }
  bool is_static() const { return body_type == RigidBodyType::Static; }
  bool is_dynamic() const { return body_type == RigidBodyType::Dynamic; }
  bool is_kinematic() const {
    return body_type == RigidBodyType::KinematicPositionBased || body_type == RigidBodyType::KinematicVelocityBased;
  }
  void accelerate(Vec2 a) { acceleration += a; }
  void apply_force(Vec2 f) {
    if (!is_static()) acceleration += f / calculated_mass;
  }
  void apply_impulse(Vec2 impulse) {
    if (!is_static()) add_velocity(impulse / calculated_mass);
  }
  void set_velocity(Vec2 v) { velocity_request = v; }
  Vec2 get_velocity() const { return calculated_velocity; }
  void add_velocity(Vec2 v) { set_velocity(get_velocity() + v); }
  void apply_force_at_point(Vec2 force, Vec2 world_point) {
    if (!is_static()) {
      apply_force(force);
      Vec2 lever = world_point - (position + center_of_mass);
      torque += lever.x * force.y - lever.y * force.x;
    }
  }
  void apply_torque_at_point(Vec2 force, Vec2 world_point) {
    if (!is_static()) {
      Vec2 lever = world_point - (position + center_of_mass);
      torque += lever.x * force.y - lever.y * force.x;
    }
  }
  void update_mass_and_inertia(const Arena<Collider>& col_set);
};

/// RigidBodyBuilder (rigid_body.rs:287-401).
class RigidBodyBuilder {
 public:
  RigidBodyBuilder& position(Vec2 p) { b_.position = p; b_.position_old = p; return *this; }
  RigidBodyBuilder& gravity_mod(float g) { b_.gravity_mod = g; return *this; }
  RigidBodyBuilder& rotation(float r) { b_.rotation = r; return *this; }
  RigidBodyBuilder& scale(Vec2 s) { b_.scale = s; return *this; }
  RigidBodyBuilder& acceleration(Vec2 a) { b_.acceleration = a; return *this; }
  RigidBodyBuilder& velocity_request(Vec2 v) { b_.velocity_request = v; return *this; }
  RigidBodyBuilder& calculated_velocity(Vec2 v) { b_.calculated_velocity = v; return *this; }
  RigidBodyBuilder& user_data(uint64_t lo, uint64_t hi = 0) { b_.user_data_lo = lo; b_.user_data_hi = hi; return *this; }
  RigidBodyBuilder& body_type(RigidBodyType t) { b_.body_type = t; return *this; }
  RigidBody build() const { return b_; }

 private:
  RigidBody b_;
};

/// Collider (collider.rs:3-71), sphere shape.  `offset` and
/// `absolute_translation` are the translations of the reference's Affine2
/// offset / absolute_transform (the only parts the step reads).
class Collider {
 public:
  Vec2 offset;
  Vec2 absolute_translation;
  uint64_t user_data_lo = 0, user_data_hi = 0;
  std::optional<RigidBodyHandle> parent;
  float radius = 0.5f;
  std::optional<float> mass_override;
  bool is_sensor = false;
  InteractionGroups collision_groups;

  float mass() const { return mass_override ? *mass_override : radius * 2.0f; }  // collider.rs:40-42
  float inertia() const {                                                         // collider.rs:44-50
    const float m = mass();
    const float d = offset.length();
    const float i = 0.5f * m * (radius * radius);
    return i + m * (d * d);
  }
};

/// ColliderBuilder (collider.rs:199-284).
class ColliderBuilder {
 public:
  ColliderBuilder& offset(Vec2 o) { c_.offset = o; return *this; }
  ColliderBuilder& absolute_translation(Vec2 t) { c_.absolute_translation = t; return *this; }
  ColliderBuilder& mass_override(float m) { c_.mass_override = m; return *this; }
  ColliderBuilder& user_data(uint64_t lo, uint64_t hi = 0) { c_.user_data_lo = lo; c_.user_data_hi = hi; return *this; }
  ColliderBuilder& parent(RigidBodyHandle p) { c_.parent = p; return *this; }
  ColliderBuilder& radius(float r) { c_.radius = r; return *this; }
  ColliderBuilder& sensor(bool s) { c_.is_sensor = s; return *this; }
  ColliderBuilder& collision_groups(InteractionGroups g) { c_.collision_groups = g; return *this; }
  Collider build() const { return c_; }

 private:
  Collider c_;
};

/// FixedJoint (joints.rs:7-19).
struct FixedJoint {
  RigidBodyHandle rigid_body_a, rigid_body_b;
  Vec2 anchor_a, anchor_b;
  float distance = 0.0f;
  float target_angle = 0.0f;
};

/// Spring (springs.rs:16-22).
struct Spring {
  RigidBodyHandle rigid_body_a, rigid_body_b;
  float rest_length = 0.0f, stiffness = 0.0f, damping = 0.0f;
};

/// Circle constraint (lib.rs:189-193).
struct Constraint {
  Vec2 position;
  float radius = 0.0f;
};

/// Physics (physics.rs:3-34).
class Physics {
 public:
  Vec2 gravity;
  uint32_t substeps = 8;
  uint32_t joint_iterations = 4;
  bool use_spatial_hash = false;
  bool collisions_enabled = true;
  double accumulator = 0.0;
  double time = 0.0;
  float old_dt = 1.0f;
  std::vector<Constraint> constraints;
  /// Axis-aligned walls (an extension without reference counterpart).
  std::optional<std::pair<Vec2, Vec2>> walls;

  explicit Physics(Vec2 gravity, bool use_spatial_hash = false, int device = 0);
  ~Physics();
  Physics(const Physics&) = delete;
  Physics& operator=(const Physics&) = delete;

  void reset();                         // physics.rs:71-76
  void step(double delta);              // physics.rs:78-82
  void fixed_step(double frame_time);   // physics.rs:84-99

  std::optional<RigidBodyData> get_rbd_data(RigidBodyHandle h);
  const RigidBody* get_rbd(RigidBodyHandle h);
  RigidBody* get_mut_rbd(RigidBodyHandle h);
  size_t rbd_count() const { return rbd_set_.len(); }
  const Collider* get_col(ColliderHandle h);

  RigidBodyHandle insert_rbd(RigidBody rbd);                                         // physics.rs:121-128
  ColliderHandle insert_collider_with_parent(Collider c, RigidBodyHandle parent);    // physics.rs:130-149
  std::optional<Vec2> rbd_position(RigidBodyHandle h);
  std::optional<Vec2> col_position(ColliderHandle h);
  void remove_col(ColliderHandle h);                                                 // physics.rs:159-161
  void remove_rbd(RigidBodyHandle h);                                                // physics.rs:163-172
  void update_rigid_body_position(uint64_t id, Vec2 offset);                         // physics.rs:174-182
  JointHandle create_fixed_joint(RigidBodyHandle a, RigidBodyHandle b, Vec2 anchor_a, Vec2 anchor_b);
  JointHandle create_fixed_joint_with_distance(RigidBodyHandle a, RigidBodyHandle b, Vec2 anchor_a, Vec2 anchor_b,
                                               float distance);
  SpringHandle insert_spring(Spring s);
  void remove_spring(SpringHandle h);

  /// Contacts counted by the contact pass since the last upload (the
  /// reference's "collisions" perf counter).
  uint64_t contact_count();

  /// collision_recv.try_iter() (physics.rs:37, :304-311): the collision
  /// events of the steps since the last call, in the reference's order.
  std::vector<CollisionEvent> collision_events();
  /// The reference's channel always receives; turning this off skips the
  /// device-side recording (and its bandwidth).
  bool record_collision_events = true;

  const Arena<RigidBody>& rbd_set() { pull(); return rbd_set_; }
  const Arena<Collider>& col_set() { pull(); return col_set_; }
  const Arena<FixedJoint>& joints() const { return joints_; }
  const Arena<Spring>& springs() const { return springs_; }

 private:
  void pull();        // device -> host when the device is newer
  void push();        // host -> device when the host is newer
  void integrate(double delta);
  Arena<RigidBody> rbd_set_;
  Arena<Collider> col_set_;
  Arena<FixedJoint> joints_;
  Arena<Spring> springs_;
  blobs_world* world_ = nullptr;
  int device_ = 0;
  void drain_events();
  bool host_dirty_ = true;     // arenas changed since the last upload
  bool device_newer_ = false;  // the device stepped since the last pull
  uint32_t event_capacity_ = 0;  // device event buffer (0: recording off)
  std::vector<CollisionEvent> events_;
  std::vector<Index> body_slots_, col_slots_;  // dense device index -> arena index
};

/// Thrown for a failed C ABI call (carries the blobs_status).
class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what)
      : std::runtime_error(what + ": " + blobs_status_string(status)), status(status) {}
  int status;
};

}  // namespace blobs
