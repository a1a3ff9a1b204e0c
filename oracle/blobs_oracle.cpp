// blobs_oracle.cpp -- TEST INFRASTRUCTURE, NOT THE PRODUCT.
//
// A CPU restatement of the reference `Physics::step` of darthdeus/blobs
// (Rust, blobs 0.2.1), used only to check results, by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  Nothing in the
// shipped library links or calls this file.
//
// The reference crate cannot be built on this machine (no Rust toolchain, the
// crates glam 0.24.2 / thunderdome 0.6.1 / bitflags 1.3.2 are not vendored),
// so this file restates the algorithm in C++ with the same operation order.
// Parity of the step itself is UNPINNED: the reference ships no test, golden
// vector or fixture for step/contacts/springs/joints/integration.  What IS
// pinned against the reference's own tests is the spatial hash
// (blobs/src/tests.rs:26-90, restated below as SpatialHash) and the body /
// collider transform composition (blobs/src/collider.rs:340-389).
//
// Two instantiations:
//   * T = float  : "f32-faithful" -- every glam Vec2 op is a scalar f32 op,
//                  compiled with -ffp-contract=off (Rust never contracts to FMA),
//                  libm sinf/cosf/atan2f as Rust std uses.
//   * T = double : the same algorithm in f64, the tolerance / finite-difference
//                  reference.
//
// Third-party arithmetic restated here (published algorithms, not copied code):
//   glam 0.24.2 Vec2: component-wise ops, dot = (x*x)+(y*y), length = sqrt(dot);
//   glam Mat2::from_angle(a) = cols [(cos a, sin a), (-sin a, cos a)];
//   glam Affine2 * Affine2: translation = M1 * t2 + t1, M*v = (m00*vx + m01*vy, m10*vx + m11*vy);
//   thunderdome Arena iteration = ascending slot order (= insertion order for a
//   world that never removed anything; the scene arrays are given in that order).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

template <class T> struct V2 {
  T x, y;
};
template <class T> inline V2<T> operator+(V2<T> a, V2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <class T> inline V2<T> operator-(V2<T> a, V2<T> b) { return {a.x - b.x, a.y - b.y}; }
template <class T> inline V2<T> operator-(V2<T> a) { return {-a.x, -a.y}; }
template <class T> inline V2<T> operator*(V2<T> a, T s) { return {a.x * s, a.y * s}; }
template <class T> inline V2<T> operator*(T s, V2<T> a) { return {s * a.x, s * a.y}; }
template <class T> inline V2<T> operator*(V2<T> a, V2<T> b) { return {a.x * b.x, a.y * b.y}; }
template <class T> inline V2<T> operator/(V2<T> a, T s) { return {a.x / s, a.y / s}; }
// glam `f32 - Vec2` broadcast, the spring quirk of blobs/src/springs.rs:41
template <class T> inline V2<T> sub_scalar_vec(T s, V2<T> a) { return {s - a.x, s - a.y}; }
template <class T> inline T dot(V2<T> a, V2<T> b) { return (a.x * b.x) + (a.y * b.y); }
template <class T> inline T length(V2<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline bool isnan2(V2<T> a) { return std::isnan(a.x) || std::isnan(a.y); }

// Rust `f32 as i32`: saturating, NaN -> 0.
template <class T> inline int32_t sat_i32(T v) {
  if (std::isnan(v)) return 0;
  if (v >= (T)2147483647.0) return 2147483647;
  if (v <= (T)-2147483648.0) return (-2147483647 - 1);
  return (int32_t)v;
}

// Affine2::from_angle_translation(theta, pos) * Affine2(offset) -> translation.
// blobs/src/rigid_body.rs:88-90 and physics.rs:360-366.
template <class T> inline V2<T> body_collider_translation(T theta, V2<T> pos, V2<T> off) {
  T s = std::sin(theta), c = std::cos(theta);
  V2<T> m = {(c * off.x) + ((-s) * off.y), (s * off.x) + (c * off.y)};
  return m + pos;
}

// ---------------------------------------------------------------------------
// SpatialHash (blobs/src/spatial.rs:31-195, HashMap variant: feature use-grid off)
// ---------------------------------------------------------------------------
struct CellHash {
  size_t operator()(const std::pair<int32_t, int32_t>& k) const {
    return std::hash<uint64_t>()(((uint64_t)(uint32_t)k.first << 32) | (uint32_t)k.second);
  }
};
struct CellPoint {
  uint64_t id;
  float x, y, radius;
};
struct SpatialHash {
  float cell_size;
  uint64_t next_id = 0;
  std::unordered_map<uint64_t, CellPoint> points;
  std::unordered_map<std::pair<int32_t, int32_t>, std::unordered_set<uint64_t>, CellHash> grid;
  std::vector<CellPoint> query_results;

  explicit SpatialHash(float cs) : cell_size(cs) {}
  // spatial.rs:57-62
  std::pair<int32_t, int32_t> cell_coords(float x, float y) const {
    return {sat_i32(std::floor(x / cell_size)), sat_i32(std::floor(y / cell_size))};
  }
  // spatial.rs:64-69
  uint64_t insert(float x, float y, float r) {
    uint64_t id = next_id++;
    insert_with_id(id, x, y, r);
    return id;
  }
  // spatial.rs:71-83
  void insert_with_id(uint64_t id, float x, float y, float r) {
    grid[cell_coords(x, y)].insert(id);
    points[id] = CellPoint{id, x, y, r};
  }
  // spatial.rs:85-100
  bool remove(uint64_t id) {
    auto it = points.find(id);
    if (it == points.end()) return false;
    auto cc = cell_coords(it->second.x, it->second.y);
    auto g = grid.find(cc);
    if (g != grid.end()) g->second.erase(id);
    points.erase(it);
    return true;
  }
  // spatial.rs:102-137
  bool move_point(uint64_t id, float dx, float dy) {
    auto it = points.find(id);
    if (it == points.end()) return false;
    float ox = it->second.x, oy = it->second.y;
    float nx = ox + dx, ny = oy + dy;
    auto oc = cell_coords(ox, oy), nc = cell_coords(nx, ny);
    if (oc != nc) {
      auto g = grid.find(oc);
      if (g != grid.end()) g->second.erase(id);
      grid[nc].insert(id);
    }
    it->second.x = nx;
    it->second.y = ny;
    return true;
  }
  // spatial.rs:139-195: 3x3 neighbour cells, filter |p-q|^2 <= (qr + r)^2
  const std::vector<CellPoint>& query(float x, float y, float qr) {
    auto cc = cell_coords(x, y);
    query_results.clear();
    const int dxs[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};
    const int dys[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
    for (int k = 0; k < 9; ++k) {
      auto g = grid.find({(int32_t)((uint32_t)cc.first + (uint32_t)dxs[k]),
                          (int32_t)((uint32_t)cc.second + (uint32_t)dys[k])});
      if (g == grid.end()) continue;
      for (uint64_t pid : g->second) {
        const CellPoint& p = points.at(pid);
        float dist = qr + p.radius;
        float ddx = p.x - x, ddy = p.y - y;
        if ((ddx * ddx) + (ddy * ddy) <= dist * dist) query_results.push_back(p);
      }
    }
    return query_results;
  }
};

}  // namespace

extern "C" {

// Scene description handed over by the test harness.  All real arrays are
// double so the f64 oracle can take perturbed parameters that f32 cannot hold;
// the f32 oracle narrows them (exact for values that came from float32).
typedef struct oracle_scene {
  double gravity[2];
  uint32_t substeps;
  uint32_t joint_iterations;
  uint32_t collisions_enabled;
  uint32_t maintain_spatial_hash;  // mirror the reference's per-body move_point cost
  uint32_t record_events;
  double old_dt;                   // physics.rs:67 initial value 1.0

  uint32_t n_bodies;
  const double* pos;          // 2n
  const double* pos_old;      // 2n, NULL -> pos
  const double* acc;          // 2n, NULL -> 0
  const double* vel;          // 2n calculated_velocity, NULL -> 0
  const double* vreq;         // 2n velocity_request value
  const uint8_t* vreq_set;    // n   velocity_request is Some
  const uint8_t* body_type;   // n   0 dynamic, 1 static, 2/3 kinematic
  const double* rotation;     // n
  const double* angvel;       // n
  const double* torque;       // n
  const double* gravity_mod;  // n, NULL -> 1
  const double* mass;         // n   calculated_mass (NULL -> computed like the reference)
  const double* inertia;      // n
  const double* bound_radius; // n   box-extension bounding radius (NULL -> computed)

  uint32_t n_colliders;
  const uint32_t* col_parent;       // c  dense body index
  const double* col_offset;         // 2c offset.translation
  const double* col_radius;         // c
  const double* col_mass_override;  // c  NaN = None; NULL -> all None
  const uint8_t* col_sensor;        // c
  const uint32_t* col_memb;         // c  InteractionGroups.memberships (NULL -> ALL)
  const uint32_t* col_filt;         // c  InteractionGroups.filter (NULL -> ALL)
  const double* col_snap;           // 2c absolute_transform.translation (NULL -> transform(body)*offset)

  uint32_t n_springs;
  const uint32_t* spr_a;
  const uint32_t* spr_b;
  const double* spr_rest;
  const double* spr_k;
  const double* spr_c;

  uint32_t n_joints;
  const uint32_t* jnt_a;
  const uint32_t* jnt_b;
  const double* jnt_anchor_a;  // 2j
  const double* jnt_anchor_b;  // 2j
  const double* jnt_distance;  // j
  const double* jnt_target;    // j  target_angle
  const uint32_t* jnt_order;   // j  processing order (NULL -> arena order)

  uint32_t n_circles;
  const double* circles;  // 3 per circle: x, y, radius  (lib.rs:189-193)

  uint32_t box_enabled;  // axis-aligned wall extension (no reference counterpart)
  double box_lo[2];
  double box_hi[2];
} oracle_scene;

enum { ORACLE_OK = 0, ORACLE_INVALID = 2, ORACLE_NAN = 4, ORACLE_GRID_PUSHOUT = 8, ORACLE_GRID_UNUSABLE = 16 };

}  // extern "C"

namespace {

// RigidBody::update_mass_and_inertia (blobs/src/rigid_body.rs:96-128) over the
// body's collider list, which the reference fills with every handle TWICE
// (collider.rs:180 and physics.rs:144).
template <class T>
void mass_and_inertia(const oracle_scene& s, std::vector<T>& mass, std::vector<T>& inertia) {
  uint32_t n = s.n_bodies;
  std::vector<std::vector<uint32_t>> lists(n);
  for (uint32_t c = 0; c < s.n_colliders; ++c) {
    lists[s.col_parent[c]].push_back(c);
    lists[s.col_parent[c]].push_back(c);
  }
  mass.assign(n, (T)1);
  inertia.assign(n, (T)1);
  for (uint32_t b = 0; b < n; ++b) {
    if (lists[b].empty()) continue;  // builder default calculated_mass 1.0, inertia 1.0
    T m = 0, I = 0;
    for (uint32_t c : lists[b]) {
      if (s.col_sensor && s.col_sensor[c]) continue;
      T r = (T)s.col_radius[c];
      T cm = (s.col_mass_override && !std::isnan(s.col_mass_override[c])) ? (T)s.col_mass_override[c]
                                                                          : r * (T)2;  // collider.rs:40-42
      V2<T> off = {(T)s.col_offset[2 * c], (T)s.col_offset[2 * c + 1]};
      T d = length(off);
      T ci = (T)0.5 * cm * (r * r);  // collider.rs:44-50
      ci = ci + cm * (d * d);
      m += cm;
      I += ci;
    }
    if (m == (T)0) m = 1;
    if (I == (T)0) I = 1;
    mass[b] = m;
    inertia[b] = I;
  }
}

struct Event {
  uint32_t a, b;
  double va[2], vb[2];
};

class WorldBase {
 public:
  virtual ~WorldBase() {}
  virtual int step(double delta) = 0;
  virtual void get_bodies(double* pos, double* pos_old, double* vel, double* rot, double* angvel) = 0;
  virtual void get_snapshots(double* snap) = 0;
  virtual void get_mass(double* mass, double* inertia) = 0;
  uint64_t contacts = 0, pushouts = 0;
  uint64_t last_substep_contacts = 0;
  double time = 0;
  std::vector<Event> events;
  // Substep trace for checking derivatives along this world's own trajectory:
  // the state at the start of every substep (position, position_old,
  // collider snapshots, calculated_velocity) and the contacts it resolved.
  bool tracing = false;
  // Enumerate contact candidates through a uniform grid (the same pairs in
  // the same order as the C^2/2 loop; for full-size checks).
  bool grid_pairs = false;
  std::vector<double> trace_states;
  std::vector<uint32_t> trace_pairs;    // (i, j | push-out << 31), collider ids, i > j
  std::vector<uint64_t> trace_counts;   // contacts per substep
};

template <class T> class World : public WorldBase {
 public:
  struct Body {
    V2<T> pos, pos_old, acc, vcalc, vreq;
    T rot, angvel, torque, inertia, mass, gmod, bound_r;
    bool has_vreq;
    uint8_t type;
    std::vector<uint32_t> colliders;  // duplicated handles, as the reference holds them
    bool is_static() const { return type == 1; }
  };
  struct Collider {
    V2<T> off, snap;
    T radius;
    bool sensor;
    uint32_t memb, filt, parent;
  };
  struct Spring {
    uint32_t a, b;
    T rest, k, c;
  };
  struct Joint {
    uint32_t a, b;
    V2<T> anchor_a, anchor_b;
    T distance, target;
  };

  V2<T> gravity;
  uint32_t substeps, joint_iterations;
  bool collisions_enabled, record_events;
  T old_dt;
  std::vector<Body> bodies;
  std::vector<Collider> cols;
  std::vector<Spring> springs;
  std::vector<Joint> joints;
  std::vector<uint32_t> joint_order;
  std::vector<T> circles;
  bool box_enabled;
  V2<T> box_lo, box_hi;
  SpatialHash* shash = nullptr;
  struct GridItem {
    V2<T> snap;
    T radius;
    uint32_t memb, filt, parent, c;
    uint64_t key;  // (row << 32) | column
  };
  std::vector<uint32_t> grid_gx, grid_gy, grid_tmp, grid_order, grid_count;
  std::vector<GridItem> grid_items;
  std::vector<uint64_t> grid_pairs_found;

  explicit World(const oracle_scene& s) {
    gravity = {(T)s.gravity[0], (T)s.gravity[1]};
    substeps = s.substeps;
    joint_iterations = s.joint_iterations;
    collisions_enabled = s.collisions_enabled != 0;
    record_events = s.record_events != 0;
    old_dt = (T)s.old_dt;
    std::vector<T> mass, inertia;
    mass_and_inertia<T>(s, mass, inertia);
    bodies.resize(s.n_bodies);
    for (uint32_t i = 0; i < s.n_bodies; ++i) {
      Body& b = bodies[i];
      b.pos = {(T)s.pos[2 * i], (T)s.pos[2 * i + 1]};
      b.pos_old = s.pos_old ? V2<T>{(T)s.pos_old[2 * i], (T)s.pos_old[2 * i + 1]} : b.pos;
      b.acc = s.acc ? V2<T>{(T)s.acc[2 * i], (T)s.acc[2 * i + 1]} : V2<T>{0, 0};
      b.vcalc = s.vel ? V2<T>{(T)s.vel[2 * i], (T)s.vel[2 * i + 1]} : V2<T>{0, 0};
      b.has_vreq = s.vreq_set ? s.vreq_set[i] != 0 : false;
      b.vreq = (s.vreq && b.has_vreq) ? V2<T>{(T)s.vreq[2 * i], (T)s.vreq[2 * i + 1]} : V2<T>{0, 0};
      b.type = s.body_type ? s.body_type[i] : 0;
      b.rot = s.rotation ? (T)s.rotation[i] : 0;
      b.angvel = s.angvel ? (T)s.angvel[i] : 0;
      b.torque = s.torque ? (T)s.torque[i] : 0;
      b.gmod = s.gravity_mod ? (T)s.gravity_mod[i] : 1;
      b.mass = s.mass ? (T)s.mass[i] : mass[i];
      b.inertia = s.inertia ? (T)s.inertia[i] : inertia[i];
      b.bound_r = s.bound_radius ? (T)s.bound_radius[i] : 0;
    }
    cols.resize(s.n_colliders);
    for (uint32_t c = 0; c < s.n_colliders; ++c) {
      Collider& k = cols[c];
      k.parent = s.col_parent[c];
      k.off = {(T)s.col_offset[2 * c], (T)s.col_offset[2 * c + 1]};
      k.radius = (T)s.col_radius[c];
      k.sensor = s.col_sensor ? s.col_sensor[c] != 0 : false;
      k.memb = s.col_memb ? s.col_memb[c] : 0xffffffffu;
      k.filt = s.col_filt ? s.col_filt[c] : 0xffffffffu;
      const Body& p = bodies[k.parent];
      k.snap = s.col_snap ? V2<T>{(T)s.col_snap[2 * c], (T)s.col_snap[2 * c + 1]}
                          : body_collider_translation(p.rot, p.pos, k.off);
      bodies[k.parent].colliders.push_back(c);
      bodies[k.parent].colliders.push_back(c);
      if (!s.bound_radius) {
        T br = length(k.off) + k.radius;
        if (br > bodies[k.parent].bound_r) bodies[k.parent].bound_r = br;
      }
    }
    springs.resize(s.n_springs);
    for (uint32_t i = 0; i < s.n_springs; ++i)
      springs[i] = Spring{s.spr_a[i], s.spr_b[i], (T)s.spr_rest[i], (T)s.spr_k[i], (T)s.spr_c[i]};
    joints.resize(s.n_joints);
    for (uint32_t i = 0; i < s.n_joints; ++i)
      joints[i] = Joint{s.jnt_a[i],
                        s.jnt_b[i],
                        {(T)s.jnt_anchor_a[2 * i], (T)s.jnt_anchor_a[2 * i + 1]},
                        {(T)s.jnt_anchor_b[2 * i], (T)s.jnt_anchor_b[2 * i + 1]},
                        (T)s.jnt_distance[i],
                        (T)s.jnt_target[i]};
    joint_order.resize(s.n_joints);
    for (uint32_t i = 0; i < s.n_joints; ++i) joint_order[i] = s.jnt_order ? s.jnt_order[i] : i;
    circles.resize(3 * s.n_circles);
    for (uint32_t i = 0; i < 3 * s.n_circles; ++i) circles[i] = (T)s.circles[i];
    box_enabled = s.box_enabled != 0;
    box_lo = {(T)s.box_lo[0], (T)s.box_lo[1]};
    box_hi = {(T)s.box_hi[0], (T)s.box_hi[1]};
    if (s.maintain_spatial_hash) {
      // Physics::new uses SpatialHash::new(2.0) (physics.rs:66); insert_rbd
      // registers each body at radius 0.5 (physics.rs:121-128).
      shash = new SpatialHash(2.0f);
      for (uint32_t i = 0; i < s.n_bodies; ++i)
        shash->insert_with_id(i, (float)bodies[i].pos.x, (float)bodies[i].pos.y, 0.5f);
    }
  }
  ~World() override { delete shash; }

  // physics.rs:369-375
  void apply_gravity() {
    for (Body& b : bodies)
      if (!b.is_static()) b.acc = b.acc + gravity * b.gmod;
  }

  // RigidBody::apply_force, rigid_body.rs:155-160
  static void apply_force(Body& b, V2<T> f) {
    if (!b.is_static()) b.acc = b.acc + f / b.mass;
  }

  // Spring::apply_force, springs.rs:25-47
  void apply_springs() {
    for (const Spring& s : springs) {
      Body& a = bodies[s.a];
      Body& b = bodies[s.b];
      V2<T> d = b.pos - a.pos;
      T dist = length(d);
      V2<T> dir = d / dist;
      V2<T> rv = a.vcalc - b.vcalc;
      V2<T> damping_force = (s.c * dot(rv, dir)) * dir;
      V2<T> fm = sub_scalar_vec(s.k * (dist - s.rest), damping_force);  // springs.rs:41 quirk
      V2<T> f = dir * fm;
      apply_force(a, f);
      apply_force(b, -f);
    }
  }

  static bool groups_test(const Collider& a, const Collider& b) {  // groups.rs:52-57
    return (a.memb & b.filt) != 0 && (b.memb & a.filt) != 0;
  }

  // One pair of the reference's contact loop (physics.rs:248-316): groups,
  // same-parent skip, f32 distance test, push-out branch, position
  // correction by mass ratio (:319-321), event.  Returns -1 if the pair is no
  // contact, 1 if it is one whose push-out moved the two snapshots, else 0 or
  // 2 for a status.
  int resolve_pair(uint32_t i, uint32_t j, uint64_t& count) {
    Collider& ca = cols[i];
    Collider& cb = cols[j];
    if (!groups_test(ca, cb)) return -1;
    if (ca.parent == cb.parent) return -1;
    V2<T> axis = ca.snap - cb.snap;
    T distance = length(axis);
    T min_dist = ca.radius + cb.radius;
    if (!(distance < min_dist)) return -1;
    Body& ra = bodies[ca.parent];
    Body& rb = bodies[cb.parent];
    const bool distance_pushed = distance < (T)1e-6f;
    if (distance_pushed) {
      V2<T> push = {(T)0.01f, (T)0};
      ra.pos = ra.pos + push;
      rb.pos = rb.pos - push;
      ca.snap = ra.pos + ca.off;
      cb.snap = rb.pos + cb.off;
      axis = ca.snap - cb.snap;
      distance = length(axis);
      ++pushouts;
    }
    V2<T> va = ra.vcalc, vb = rb.vcalc;
    if (!ca.sensor && !cb.sensor) {
      V2<T> n = axis / distance;
      if (isnan2(n)) return 2 + ORACLE_NAN;  // physics.rs:293 assert
      T delta = min_dist - distance;
      T ratio = (T)1 - ra.mass / (ra.mass + rb.mass);
      ra.pos = ra.pos + (ratio * delta) * n;
      rb.pos = rb.pos - (((T)1 - ratio) * delta) * n;
    }
    ++count;
    if (tracing) {
      trace_pairs.push_back(i);
      trace_pairs.push_back(j | (distance_pushed ? 0x80000000u : 0u));
    }
    if (record_events) events.push_back(Event{i, j, {(double)va.x, (double)va.y}, {(double)vb.x, (double)vb.y}});
    return distance_pushed ? 1 : 0;
  }

  // physics.rs:241-317: every collider pair (i, j < i) in arena order.
  int brute_force_collisions() {
    uint64_t count = 0;
    const uint32_t nc = (uint32_t)cols.size();
    if (grid_pairs) {
      int st = grid_collisions(count);
      if (st != ORACLE_GRID_UNUSABLE) return finish_collisions(count, st);
      count = 0;
    }
    for (uint32_t i = 0; i < nc; ++i) {
      // the rejection tests of resolve_pair inline, so the C^2/2 loop pays
      // for the call only on contacts (it repeats them on the same values)
      const uint32_t memb = cols[i].memb, filt = cols[i].filt, parent = cols[i].parent;
      const T radius = cols[i].radius;
      V2<T> snap = cols[i].snap;
      for (uint32_t j = 0; j < i; ++j) {
        const Collider& cb = cols[j];
        if (!((memb & cb.filt) != 0 && (cb.memb & filt) != 0) || parent == cb.parent) continue;
        if (!(length(snap - cb.snap) < radius + cb.radius)) continue;
        int r = resolve_pair(i, j, count);
        if (r >= 2) return r - 2;
        snap = cols[i].snap;  // a push-out refreshes collider i's snapshot
      }
    }
    return finish_collisions(count, ORACLE_OK);
  }

  int finish_collisions(uint64_t count, int st) {
    contacts += count;
    last_substep_contacts = count;
    if (tracing) trace_counts.push_back(count);
    return st;
  }

  // The same pairs in the same order, enumerated through a uniform grid of
  // the substep's collider snapshots instead of all C^2/2 pairs.  A contact
  // needs |snap_i - snap_j| < r_i + r_j <= 2 r_max, and the cell edge is
  // 2 r_max (1 + 2^-6), so every contact's partner lies in the 3x3 cells
  // around a collider.  The colliders are counting-sorted by (row, column);
  // a sweep in that order keeps, for each of the three neighbour rows, the
  // range of the three neighbour cells with pointers that only move forward.
  // The contacts found are then resolved in the reference's order: i
  // ascending, j < i ascending.
  // Returns ORACLE_GRID_UNUSABLE before touching any state when the grid does
  // not fit (non-finite snapshots, more rows plus columns than 64 per
  // collider), and ORACLE_GRID_PUSHOUT if a push-out moved two snapshots (the
  // grid is then stale; the caller must not use this mode on such scenes).
  int grid_collisions(uint64_t& count) {
    const uint32_t nc = (uint32_t)cols.size();
    if (nc < 2) return ORACLE_OK;
    double rmax = 0, lo[2] = {HUGE_VAL, HUGE_VAL}, hi[2] = {-HUGE_VAL, -HUGE_VAL};
    for (const Collider& c : cols) {
      const double x = (double)c.snap.x, y = (double)c.snap.y;
      if (!std::isfinite(x) || !std::isfinite(y) || !std::isfinite((double)c.radius)) return ORACLE_GRID_UNUSABLE;
      rmax = std::fmax(rmax, (double)c.radius);
      lo[0] = std::fmin(lo[0], x), lo[1] = std::fmin(lo[1], y);
      hi[0] = std::fmax(hi[0], x), hi[1] = std::fmax(hi[1], y);
    }
    const double cs = rmax > 0 ? 2.0 * rmax * (1.0 + 1.0 / 64.0) : 1.0;
    const double wd = std::floor((hi[0] - lo[0]) / cs) + 1, hd = std::floor((hi[1] - lo[1]) / cs) + 1;
    if (!(wd + hd <= 64.0 * nc + 65536.0)) return ORACLE_GRID_UNUSABLE;
    const uint32_t W = (uint32_t)wd, H = (uint32_t)hd;
    // cell coordinates, then a stable counting sort by column and one by row
    grid_gx.resize(nc), grid_gy.resize(nc), grid_tmp.resize(nc), grid_order.resize(nc);
    for (uint32_t c = 0; c < nc; ++c) {
      const uint32_t gx = (uint32_t)std::floor(((double)cols[c].snap.x - lo[0]) / cs);
      const uint32_t gy = (uint32_t)std::floor(((double)cols[c].snap.y - lo[1]) / cs);
      grid_gx[c] = gx < W ? gx : W - 1, grid_gy[c] = gy < H ? gy : H - 1;
    }
    auto counting_sort = [&](const std::vector<uint32_t>& key, uint32_t range, const std::vector<uint32_t>& in,
                             std::vector<uint32_t>& out) {
      grid_count.assign((size_t)range + 1, 0);
      for (uint32_t c : in) ++grid_count[key[c] + 1];
      for (uint32_t k = 0; k < range; ++k) grid_count[k + 1] += grid_count[k];
      for (uint32_t c : in) out[grid_count[key[c]]++] = c;
    };
    for (uint32_t c = 0; c < nc; ++c) grid_tmp[c] = c;
    counting_sort(grid_gx, W, grid_tmp, grid_order);
    counting_sort(grid_gy, H, grid_order, grid_tmp);
    // candidate records in (row, column) order, so the sweep streams them
    grid_items.resize(nc);
    for (uint32_t q = 0; q < nc; ++q) {
      const uint32_t c = grid_tmp[q];
      const Collider& k = cols[c];
      grid_items[q] = GridItem{k.snap, k.radius, k.memb, k.filt, k.parent, c,
                               ((uint64_t)grid_gy[c] << 32) | grid_gx[c]};
    }
    grid_pairs_found.clear();
    uint32_t first[3] = {0, 0, 0}, last[3] = {0, 0, 0};  // per neighbour row: [first, last) of its 3 cells
    for (uint32_t q = 0; q < nc; ++q) {
      const GridItem& gi = grid_items[q];
      const uint32_t i = gi.c;
      const uint64_t gy = gi.key >> 32, gx = gi.key & 0xffffffffu;
      for (int r = 0; r < 3; ++r) {
        if (gy + r < 1) continue;  // the row below row 0
        const uint64_t row = gy + r - 1;
        const uint64_t k0 = (row << 32) | (gx ? gx - 1 : 0), k1 = (row << 32) | (gx + 1);
        while (first[r] < nc && grid_items[first[r]].key < k0) ++first[r];
        if (last[r] < first[r]) last[r] = first[r];
        while (last[r] < nc && grid_items[last[r]].key <= k1) ++last[r];
        for (uint32_t k = first[r]; k < last[r]; ++k) {
          const GridItem& g = grid_items[k];
          if (g.c >= i) continue;
          // the same test resolve_pair makes; it is repeated there on the
          // unchanged snapshots, so this only drops pairs that are no contact
          if (!((gi.memb & g.filt) != 0 && (g.memb & gi.filt) != 0) || gi.parent == g.parent) continue;
          const V2<T> axis = gi.snap - g.snap;
          const T min_dist = gi.radius + g.radius;
          // far pairs leave before the square root: sqrt rounds by at most
          // half an ulp, so dot >= (1 + 2^-20) min_dist^2 means length >= min_dist
          if ((double)dot(axis, axis) >= (double)min_dist * (double)min_dist * (1.0 + 0x1p-20)) continue;
          if (!(length(axis) < min_dist)) continue;
          grid_pairs_found.push_back(((uint64_t)i << 32) | g.c);
        }
      }
    }
    std::sort(grid_pairs_found.begin(), grid_pairs_found.end());
    for (uint64_t key : grid_pairs_found) {
      int r = resolve_pair((uint32_t)(key >> 32), (uint32_t)key, count);
      if (r == 1) return ORACLE_GRID_PUSHOUT;
      if (r >= 2) return r - 2;
    }
    return ORACLE_OK;
  }

  // physics.rs:424-477
  int solve_fixed_joints(T dt) {
    for (uint32_t it = 0; it < joint_iterations; ++it) {
      for (uint32_t q = 0; q < joints.size(); ++q) {
        const Joint& j = joints[joint_order[q]];
        Body& a = bodies[j.a];
        Body& b = bodies[j.b];
        V2<T> wa = a.pos + j.anchor_a;
        V2<T> wb = b.pos + j.anchor_b;
        V2<T> dp = wb - wa;
        T distance = length(dp);
        if (distance < (T)1e-6f) continue;
        T off_by = distance - j.distance;
        V2<T> correction = (off_by * dp) / distance;
        if (!(a.mass > 0) || !(b.mass > 0)) return ORACLE_INVALID;
        T ims = ((T)1 / a.mass) + ((T)1 / b.mass);
        if (a.is_static()) {
          b.pos = b.pos - ims * correction;
        } else if (b.is_static()) {
          a.pos = a.pos + ims * correction;
        } else {
          T ratio = ((T)1 / a.mass) / ims;
          a.pos = a.pos + ratio * correction;
          b.pos = b.pos - ((T)1 - ratio) * correction;
        }
        T angle_a = std::atan2(dp.y, dp.x);
        T angle_b = -std::atan2(dp.y, -dp.x);  // physics.rs:464 precedence
        T angle_diff = (angle_b - angle_a) - j.target;
        T rc = angle_diff * (T)0.5;
        a.rot = a.rot + rc * dt;
        b.rot = b.rot - rc * dt;
        if (!std::isfinite(a.rot) || !std::isfinite(b.rot)) return ORACLE_NAN;
      }
    }
    return ORACLE_OK;
  }

  // physics.rs:323-367
  void update_objects(T dt) {
    for (uint32_t i = 0; i < bodies.size(); ++i) {
      Body& b = bodies[i];
      if (b.is_static()) {
        b.pos_old = b.pos;
        b.acc = {0, 0};
        b.vcalc = {0, 0};
        continue;
      }
      if (b.has_vreq) {
        b.pos_old = b.pos - b.vreq * dt;
        b.has_vreq = false;
      }
      V2<T> disp = (b.pos - b.pos_old) * (dt / old_dt);
      old_dt = dt;
      if (shash) shash->move_point(i, (float)disp.x, (float)disp.y);
      b.pos_old = b.pos;
      b.pos = b.pos + (disp + (b.acc * dt) * dt);
      b.angvel = b.angvel + (b.torque / b.inertia) * dt;
      b.rot = b.rot + b.angvel * dt;
      b.torque = 0;
      b.acc = {0, 0};
      b.vcalc = disp / dt;
    }
    for (Body& b : bodies)
      for (uint32_t c : b.colliders) cols[c].snap = body_collider_translation(b.rot, b.pos, cols[c].off);
  }

  // physics.rs:377-395, then the axis-aligned wall extension.
  void apply_constraints() {
    for (size_t k = 0; k < circles.size() / 3; ++k) {
      V2<T> c = {circles[3 * k], circles[3 * k + 1]};
      T radius = circles[3 * k + 2];
      for (Body& b : bodies) {
        V2<T> to = b.pos - c;
        T dist = length(to);
        if (dist > radius) {
          V2<T> n = to / dist;
          b.pos = c + n * radius;
        }
      }
    }
    if (box_enabled) {
      for (Body& b : bodies) {
        b.pos.x = std::fmin(std::fmax(b.pos.x, box_lo.x + b.bound_r), box_hi.x - b.bound_r);
        b.pos.y = std::fmin(std::fmax(b.pos.y, box_lo.y + b.bound_r), box_hi.y - b.bound_r);
      }
    }
  }

  // physics.rs:397-422
  int integrate(uint32_t n_sub, T delta) {
    T step_delta = delta / (T)n_sub;
    for (uint32_t s = 0; s < n_sub; ++s) {
      if (tracing) trace_state();
      if (tracing && !collisions_enabled) trace_counts.push_back(0);
      apply_gravity();
      apply_springs();
      if (collisions_enabled) {
        int st = brute_force_collisions();
        if (st) return st;
      }
      int st = solve_fixed_joints(step_delta);
      if (st) return st;
      update_objects(step_delta);
      apply_constraints();
    }
    return ORACLE_OK;
  }

  void trace_state() {
    for (const Body& b : bodies) trace_states.push_back((double)b.pos.x), trace_states.push_back((double)b.pos.y);
    for (const Body& b : bodies)
      trace_states.push_back((double)b.pos_old.x), trace_states.push_back((double)b.pos_old.y);
    for (const Collider& c : cols) trace_states.push_back((double)c.snap.x), trace_states.push_back((double)c.snap.y);
    for (const Body& b : bodies) trace_states.push_back((double)b.vcalc.x), trace_states.push_back((double)b.vcalc.y);
  }

  // physics.rs:78-82
  int step(double delta) override {
    int st = integrate(substeps, (T)delta);
    time += delta;
    return st;
  }

  void get_bodies(double* pos, double* pos_old, double* vel, double* rot, double* angvel) override {
    for (size_t i = 0; i < bodies.size(); ++i) {
      const Body& b = bodies[i];
      if (pos) pos[2 * i] = b.pos.x, pos[2 * i + 1] = b.pos.y;
      if (pos_old) pos_old[2 * i] = b.pos_old.x, pos_old[2 * i + 1] = b.pos_old.y;
      if (vel) vel[2 * i] = b.vcalc.x, vel[2 * i + 1] = b.vcalc.y;
      if (rot) rot[i] = b.rot;
      if (angvel) angvel[i] = b.angvel;
    }
  }
  void get_snapshots(double* snap) override {
    for (size_t c = 0; c < cols.size(); ++c) snap[2 * c] = cols[c].snap.x, snap[2 * c + 1] = cols[c].snap.y;
  }
  void get_mass(double* mass, double* inertia) override {
    for (size_t i = 0; i < bodies.size(); ++i) {
      if (mass) mass[i] = bodies[i].mass;
      if (inertia) inertia[i] = bodies[i].inertia;
    }
  }
};

}  // namespace

extern "C" {

// precision: 32 -> f32-faithful, 64 -> f64
void* oracle_world_new(const oracle_scene* s, int precision) {
  if (precision == 64) return static_cast<WorldBase*>(new World<double>(*s));
  return static_cast<WorldBase*>(new World<float>(*s));
}
void oracle_world_free(void* w) { delete static_cast<WorldBase*>(w); }
int oracle_world_step(void* w, double delta, uint32_t n_steps) {
  WorldBase* wb = static_cast<WorldBase*>(w);
  for (uint32_t i = 0; i < n_steps; ++i) {
    int st = wb->step(delta);
    if (st) return st;
  }
  return ORACLE_OK;
}
// Wall-clock seconds for n_steps of step(delta) (CPU-baseline leg).
double oracle_world_time_steps(void* w, double delta, uint32_t n_steps, int* status) {
  auto t0 = std::chrono::steady_clock::now();
  int st = oracle_world_step(w, delta, n_steps);
  auto t1 = std::chrono::steady_clock::now();
  if (status) *status = st;
  return std::chrono::duration<double>(t1 - t0).count();
}
void oracle_world_get_bodies(void* w, double* pos, double* pos_old, double* vel, double* rot, double* angvel) {
  static_cast<WorldBase*>(w)->get_bodies(pos, pos_old, vel, rot, angvel);
}
void oracle_world_get_snapshots(void* w, double* snap) { static_cast<WorldBase*>(w)->get_snapshots(snap); }
void oracle_world_get_mass(void* w, double* mass, double* inertia) {
  static_cast<WorldBase*>(w)->get_mass(mass, inertia);
}
uint64_t oracle_world_contacts(void* w) { return static_cast<WorldBase*>(w)->contacts; }
uint64_t oracle_world_last_substep_contacts(void* w) { return static_cast<WorldBase*>(w)->last_substep_contacts; }
uint64_t oracle_world_pushouts(void* w) { return static_cast<WorldBase*>(w)->pushouts; }
double oracle_world_time(void* w) { return static_cast<WorldBase*>(w)->time; }
uint64_t oracle_world_events(void* w, uint32_t* a, uint32_t* b, double* va, double* vb, uint64_t cap) {
  WorldBase* wb = static_cast<WorldBase*>(w);
  uint64_t n = wb->events.size() < cap ? wb->events.size() : cap;
  for (uint64_t i = 0; i < n; ++i) {
    const Event& e = wb->events[i];
    a[i] = e.a;
    b[i] = e.b;
    va[2 * i] = e.va[0], va[2 * i + 1] = e.va[1];
    vb[2 * i] = e.vb[0], vb[2 * i + 1] = e.vb[1];
  }
  return wb->events.size();
}
void oracle_world_clear_events(void* w) { static_cast<WorldBase*>(w)->events.clear(); }
void oracle_world_set_grid_pairs(void* w, int on) { static_cast<WorldBase*>(w)->grid_pairs = on != 0; }

// Substep trace (test infrastructure for derivative checks): on != 0 clears
// and starts it.  Each state is 2n position, 2n position_old, 2c snapshots,
// 2n calculated_velocity, recorded at the start of every substep.
void oracle_world_trace(void* w, int on) {
  WorldBase* wb = static_cast<WorldBase*>(w);
  wb->tracing = on != 0;
  wb->trace_states.clear();
  wb->trace_pairs.clear();
  wb->trace_counts.clear();
}
uint64_t oracle_world_trace_states(void* w, double* out, uint64_t cap) {
  const std::vector<double>& v = static_cast<WorldBase*>(w)->trace_states;
  for (uint64_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
  return v.size();
}
uint64_t oracle_world_trace_pairs(void* w, uint32_t* out, uint64_t cap) {
  const std::vector<uint32_t>& v = static_cast<WorldBase*>(w)->trace_pairs;
  for (uint64_t i = 0; i < v.size() && i < 2 * cap; ++i) out[i] = v[i];
  return v.size() / 2;
}
uint64_t oracle_world_trace_counts(void* w, uint64_t* out, uint64_t cap) {
  const std::vector<uint64_t>& v = static_cast<WorldBase*>(w)->trace_counts;
  for (uint64_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
  return v.size();
}

// update_mass_and_inertia over a whole scene (f32), rigid_body.rs:96-128.
void oracle_mass_inertia_f32(const oracle_scene* s, float* mass, float* inertia) {
  std::vector<float> m, I;
  mass_and_inertia<float>(*s, m, I);
  for (uint32_t i = 0; i < s->n_bodies; ++i) mass[i] = m[i], inertia[i] = I[i];
}

// Body transform composed with a collider offset, f32 (rigid_body.rs:88-90,
// collider.rs:340-389): out = {m00, m10, m01, m11, tx, ty}.
void oracle_body_collider_transform(float theta, float px, float py, float ox, float oy, float* out) {
  float s = std::sin(theta), c = std::cos(theta);
  out[0] = c, out[1] = s, out[2] = -s, out[3] = c;
  V2<float> t = body_collider_translation<float>(theta, {px, py}, {ox, oy});
  out[4] = t.x, out[5] = t.y;
}

// The reference's O(C^2/2) contact detection alone, f32: emits the contact
// pairs (i > j, sequence order) of one brute_force_collisions pass without
// moving anything.  Used to check the GPU broadphase + narrowphase pair set.
uint64_t oracle_contact_pairs(uint32_t n, const float* snap, const float* radius, const uint32_t* parent,
                              const uint32_t* memb, const uint32_t* filt, uint32_t* out_i, uint32_t* out_j,
                              uint64_t cap) {
  uint64_t k = 0;
  for (uint32_t i = 0; i < n; ++i)
    for (uint32_t j = 0; j < i; ++j) {
      uint32_t mi = memb ? memb[i] : 0xffffffffu, fi = filt ? filt[i] : 0xffffffffu;
      uint32_t mj = memb ? memb[j] : 0xffffffffu, fj = filt ? filt[j] : 0xffffffffu;
      if (!((mi & fj) != 0 && (mj & fi) != 0)) continue;
      if (parent && parent[i] == parent[j]) continue;
      V2<float> axis = {snap[2 * i] - snap[2 * j], snap[2 * i + 1] - snap[2 * j + 1]};
      float d = length(axis);
      if (d < radius[i] + radius[j]) {
        if (k < cap) out_i[k] = i, out_j[k] = j;
        ++k;
      }
    }
  return k;
}

// ---- SpatialHash (spatial.rs) for the reference's own known-answer tests ----
void* oracle_sh_new(float cell_size) { return new SpatialHash(cell_size); }
void oracle_sh_free(void* h) { delete static_cast<SpatialHash*>(h); }
uint64_t oracle_sh_insert(void* h, float x, float y, float r) { return static_cast<SpatialHash*>(h)->insert(x, y, r); }
void oracle_sh_insert_with_id(void* h, uint64_t id, float x, float y, float r) {
  static_cast<SpatialHash*>(h)->insert_with_id(id, x, y, r);
}
int oracle_sh_remove(void* h, uint64_t id) { return static_cast<SpatialHash*>(h)->remove(id) ? 1 : 0; }
int oracle_sh_move_point(void* h, uint64_t id, float dx, float dy) {
  return static_cast<SpatialHash*>(h)->move_point(id, dx, dy) ? 1 : 0;
}
void oracle_sh_cell_coords(void* h, float x, float y, int32_t* cx, int32_t* cy) {
  auto c = static_cast<SpatialHash*>(h)->cell_coords(x, y);
  *cx = c.first, *cy = c.second;
}
uint64_t oracle_sh_next_id(void* h) { return static_cast<SpatialHash*>(h)->next_id; }
int oracle_sh_point(void* h, uint64_t id, float* x, float* y) {
  SpatialHash* sh = static_cast<SpatialHash*>(h);
  auto it = sh->points.find(id);
  if (it == sh->points.end()) return 0;
  *x = it->second.x, *y = it->second.y;
  return 1;
}
uint64_t oracle_sh_cell_len(void* h, int32_t cx, int32_t cy) {
  SpatialHash* sh = static_cast<SpatialHash*>(h);
  auto g = sh->grid.find({cx, cy});
  return g == sh->grid.end() ? (uint64_t)-1 : (uint64_t)g->second.size();
}
uint64_t oracle_sh_query(void* h, float x, float y, float qr, uint64_t* ids, float* pos, uint64_t cap) {
  const auto& r = static_cast<SpatialHash*>(h)->query(x, y, qr);
  for (size_t i = 0; i < r.size() && i < cap; ++i) {
    ids[i] = r[i].id;
    pos[2 * i] = r[i].x, pos[2 * i + 1] = r[i].y;
  }
  return r.size();
}

}  // extern "C"
