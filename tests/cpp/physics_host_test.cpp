// Test driver of the C++ host mirror (include/blobs_physics.hpp).
//   physics_host_test cpu                      arena / builder / mass semantics (no device)
//   physics_host_test scene IN OUT STEPS DT    build a world through the Physics API the way the
//                                              reference demo does (demo/src/simulation.rs:99-146),
//                                              step it on the GPU, write the body state
//   physics_host_test mutate IN OUT S1 S2 DT K  the same world: S1 steps, then remove_rbd of every
//                                              K-th body and remove_col of the collider of every
//                                              K-th body after it (physics.rs:159-172), S2 steps
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "blobs_physics.hpp"

using namespace blobs;

static int failures = 0;
#define EXPECT(cond)                                                  \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                     \
    }                                                                 \
  } while (0)

static int cpu_tests() {
  // thunderdome semantics: generation bumps on removal, LIFO slot reuse
  Arena<int> a;
  Index i0 = a.insert(10), i1 = a.insert(11), i2 = a.insert(12);
  EXPECT(i0.slot == 0 && i1.slot == 1 && i2.slot == 2 && i0.generation == 1);
  EXPECT(a.remove(i1).value() == 11);
  EXPECT(!a.contains(i1) && a.len() == 2);
  Index i3 = a.insert(13);
  EXPECT(i3.slot == 1 && i3.generation == 2 && a.get(i1) == nullptr && *a.get(i3) == 13);
  EXPECT(Index::from_bits(i3.to_bits()) == i3);
  std::vector<int> order;
  a.for_each([&](Index, int v) { order.push_back(v); });
  EXPECT(order.size() == 3 && order[0] == 10 && order[1] == 13 && order[2] == 12);

  // builder defaults (rigid_body.rs:303-318, :376-400)
  RigidBody b = RigidBodyBuilder().position(Vec2(2, 3)).build();
  EXPECT(b.position == Vec2(2, 3) && b.position_old == Vec2(2, 3) && b.calculated_mass == 1.0f &&
         b.inertia == 1.0f && b.gravity_mod == 1.0f && !b.velocity_request);

  // doubled collider registration: mass 4r, inertia 2 * (0.5 * 2r * r^2)
  Physics p(Vec2(0, -9.81f));
  RigidBodyHandle h = p.insert_rbd(RigidBodyBuilder().position(Vec2(0, 0)).build());
  ColliderHandle c = p.insert_collider_with_parent(ColliderBuilder().radius(0.25f).build(), h);
  const RigidBody* rb = p.get_rbd(h);
  EXPECT(rb->colliders.size() == 2 && rb->colliders[0] == c && rb->colliders[1] == c);
  EXPECT(rb->calculated_mass == 1.0f);
  EXPECT(rb->inertia == 2.0f * (0.5f * 0.5f * (0.25f * 0.25f)));
  // a second collider with an offset
  p.insert_collider_with_parent(ColliderBuilder().radius(0.5f).offset(Vec2(3, 4)).build(), h);
  EXPECT(p.get_rbd(h)->calculated_mass == 1.0f + 2.0f);
  // sensors do not weigh
  RigidBodyHandle hs = p.insert_rbd(RigidBodyBuilder().build());
  p.insert_collider_with_parent(ColliderBuilder().radius(0.3f).sensor(true).build(), hs);
  EXPECT(p.get_rbd(hs)->calculated_mass == 1.0f);

  // fixed joint: distance = |pa + aa - pb - ab|, target = rot_b - rot_a (physics.rs:198, :230)
  RigidBodyHandle h2 = p.insert_rbd(RigidBodyBuilder().position(Vec2(3, 4)).rotation(0.5f).build());
  JointHandle j = p.create_fixed_joint(h, h2, Vec2(0, 0), Vec2(0, 0));
  const FixedJoint* fj = p.joints().get(j.idx);
  EXPECT(fj && fj->distance == 5.0f && fj->target_angle == 0.5f);
  EXPECT(p.get_rbd(h)->connected_joints.size() == 1 && p.get_rbd(h2)->connected_joints.size() == 1);

  // remove_col drops the body once its last collider is gone (collider.rs:143-158)
  EXPECT(p.rbd_count() == 3);
  RigidBodyHandle h3 = p.insert_rbd(RigidBodyBuilder().build());
  ColliderHandle c3 = p.insert_collider_with_parent(ColliderBuilder().build(), h3);
  p.remove_col(c3);
  EXPECT(p.get_rbd(h3) == nullptr && p.get_col(c3) == nullptr);
  // remove_rbd removes the body's colliders
  p.remove_rbd(h);
  EXPECT(p.get_col(c) == nullptr && p.get_rbd(h) == nullptr);

  // update_rigid_body_position (physics.rs:174-182)
  p.update_rigid_body_position(h2.idx.to_bits(), Vec2(1, 1));
  EXPECT(*p.rbd_position(h2) == Vec2(4, 5));

  // missing parent -> error instead of the reference's panic (physics.rs:142)
  bool threw = false;
  try {
    p.insert_collider_with_parent(ColliderBuilder().build(), h);
  } catch (const Error& e) {
    threw = e.status == BLOBS_ERR_INVALID_HANDLE;
  }
  EXPECT(threw);
  std::printf("cpu tests: %d failures\n", failures);
  return failures ? 1 : 0;
}

// IN: u32 n, f32 gravity[2], f32 box[4], then per body: pos[2], vel[2], radius, u8 type
// OUT: per body pos[2], pos_old[2], vel[2]; then u64 contacts; then u64
// events and per event u32 collider slot a, b, f32 impact_vel_a[2], _b[2]
static int scene_test(const char* in, const char* out, int steps, double dt) {
  FILE* f = std::fopen(in, "rb");
  if (!f) return 2;
  uint32_t n;
  float g[2], box[4];
  if (std::fread(&n, 4, 1, f) != 1 || std::fread(g, 4, 2, f) != 2 || std::fread(box, 4, 4, f) != 4) return 2;
  Physics p(Vec2(g[0], g[1]));
  p.walls = std::make_pair(Vec2(box[0], box[1]), Vec2(box[2], box[3]));
  std::vector<RigidBodyHandle> hs;
  for (uint32_t i = 0; i < n; ++i) {
    float rec[5];
    uint8_t type;
    if (std::fread(rec, 4, 5, f) != 5 || std::fread(&type, 1, 1, f) != 1) return 2;
    RigidBodyHandle h = p.insert_rbd(RigidBodyBuilder()
                                         .position(Vec2(rec[0], rec[1]))
                                         .velocity_request(Vec2(rec[2], rec[3]))
                                         .body_type((RigidBodyType)type)
                                         .build());
    p.insert_collider_with_parent(
        ColliderBuilder().radius(rec[4]).absolute_translation(Vec2(rec[0], rec[1])).build(), h);
    hs.push_back(h);
  }
  std::fclose(f);
  std::vector<CollisionEvent> events;
  for (int s = 0; s < steps; ++s) {
    p.step(dt);
    std::vector<CollisionEvent> e = p.collision_events();
    events.insert(events.end(), e.begin(), e.end());
  }
  FILE* o = std::fopen(out, "wb");
  for (RigidBodyHandle h : hs) {
    const RigidBody* b = p.get_rbd(h);
    float rec[6] = {b->position.x, b->position.y, b->position_old.x, b->position_old.y, b->calculated_velocity.x,
                    b->calculated_velocity.y};
    std::fwrite(rec, 4, 6, o);
  }
  uint64_t contacts = p.contact_count();
  std::fwrite(&contacts, 8, 1, o);
  const uint64_t n_events = events.size();
  std::fwrite(&n_events, 8, 1, o);
  for (const CollisionEvent& e : events) {
    const uint32_t ab[2] = {e.col_handle_a.idx.slot, e.col_handle_b.idx.slot};
    const float v[4] = {e.impact_vel_a.x, e.impact_vel_a.y, e.impact_vel_b.x, e.impact_vel_b.y};
    std::fwrite(ab, 4, 2, o);
    std::fwrite(v, 4, 4, o);
  }
  std::fclose(o);
  return 0;
}

// IN as for scene_test.  OUT: the state of every body after S1 steps (pos,
// pos_old, vel, snapshot: 8 floats), then the state of the remaining bodies
// after S2 more steps (same 8 floats each).
static int mutate_test(const char* in, const char* out, int s1, int s2, double dt, int every) {
  FILE* f = std::fopen(in, "rb");
  if (!f) return 2;
  uint32_t n;
  float g[2], box[4];
  if (std::fread(&n, 4, 1, f) != 1 || std::fread(g, 4, 2, f) != 2 || std::fread(box, 4, 4, f) != 4) return 2;
  Physics p(Vec2(g[0], g[1]));
  p.walls = std::make_pair(Vec2(box[0], box[1]), Vec2(box[2], box[3]));
  std::vector<RigidBodyHandle> hs;
  std::vector<ColliderHandle> cs;
  for (uint32_t i = 0; i < n; ++i) {
    float rec[5];
    uint8_t type;
    if (std::fread(rec, 4, 5, f) != 5 || std::fread(&type, 1, 1, f) != 1) return 2;
    RigidBodyHandle h = p.insert_rbd(RigidBodyBuilder()
                                         .position(Vec2(rec[0], rec[1]))
                                         .velocity_request(Vec2(rec[2], rec[3]))
                                         .body_type((RigidBodyType)type)
                                         .build());
    cs.push_back(p.insert_collider_with_parent(
        ColliderBuilder().radius(rec[4]).absolute_translation(Vec2(rec[0], rec[1])).build(), h));
    hs.push_back(h);
  }
  std::fclose(f);
  FILE* o = std::fopen(out, "wb");
  auto dump = [&](uint32_t i) {
    const RigidBody* b = p.get_rbd(hs[i]);
    const Collider* c = p.get_col(cs[i]);
    float rec[8] = {b->position.x, b->position.y, b->position_old.x, b->position_old.y,
                    b->calculated_velocity.x, b->calculated_velocity.y, c->absolute_translation.x,
                    c->absolute_translation.y};
    std::fwrite(rec, 4, 8, o);
  };
  for (int s = 0; s < s1; ++s) p.step(dt);
  for (uint32_t i = 0; i < n; ++i) dump(i);
  std::vector<bool> gone(n, false);
  for (uint32_t i = 0; i < n; i += (uint32_t)every) {
    p.remove_rbd(hs[i]);
    gone[i] = true;
    if (i + 1 < n) {
      p.remove_col(cs[i + 1]);  // the body's last collider: the body goes too
      gone[i + 1] = true;
    }
  }
  for (int s = 0; s < s2; ++s) p.step(dt);
  for (uint32_t i = 0; i < n; ++i) {
    EXPECT(gone[i] == (p.get_rbd(hs[i]) == nullptr));
    if (!gone[i]) dump(i);
  }
  std::fclose(o);
  return failures ? 1 : 0;
}

int main(int argc, char** argv) {
  try {
    if (argc >= 2 && std::strcmp(argv[1], "cpu") == 0) return cpu_tests();
    if (argc >= 6 && std::strcmp(argv[1], "scene") == 0)
      return scene_test(argv[2], argv[3], std::atoi(argv[4]), std::atof(argv[5]));
    if (argc >= 8 && std::strcmp(argv[1], "mutate") == 0)
      return mutate_test(argv[2], argv[3], std::atoi(argv[4]), std::atoi(argv[5]), std::atof(argv[6]),
                         std::atoi(argv[7]));
  } catch (const Error& e) {
    std::fprintf(stderr, "blobs error: %s\n", e.what());
    return 3;
  }
  std::fprintf(stderr, "usage: %s cpu | scene IN OUT STEPS DT | mutate IN OUT S1 S2 DT K\n", argv[0]);
  return 2;
}
