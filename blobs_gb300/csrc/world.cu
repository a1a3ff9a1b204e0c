// world.cu -- host side of the device world behind include/blobs_gpu.h.
//
// A blobs_world holds one scene (one reference `Physics`, or a batch of
// independent ones packed back to back) resident in HBM as
// structure-of-arrays, a CUDA stream, and the CUDA graphs of its steps.
// `step(dt)` (physics.rs:78-82) is one graph launch of `substeps` substeps.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <numeric>
#include <vector>

#include "blobs_gpu.h"
#include "device.cuh"
#include "kernels.h"
#include "world.h"

using namespace blobs;

namespace {

struct Counters {
  unsigned long long contacts_total[COUNTER_BINS];
  unsigned long long pushouts_total[COUNTER_BINS];
  uint32_t contacts_sub[COUNTER_BINS];
  unsigned long long defer_total[COUNTER_BINS];
  uint32_t defer_sub[COUNTER_BINS];
  uint32_t status;
  uint32_t pad[3];
  unsigned long long contacts() const {
    unsigned long long t = 0;
    for (uint32_t i = 0; i < COUNTER_BINS; ++i) t += contacts_total[i];
    return t;
  }
  unsigned long long deferred() const {
    unsigned long long t = 0;
    for (uint32_t i = 0; i < COUNTER_BINS; ++i) t += defer_total[i];
    return t;
  }
  unsigned long long deferred_sub() const {
    unsigned long long t = 0;
    for (uint32_t i = 0; i < COUNTER_BINS; ++i) t += defer_sub[i];
    return t;
  }
  unsigned long long pushouts() const {
    unsigned long long t = 0;
    for (uint32_t i = 0; i < COUNTER_BINS; ++i) t += pushouts_total[i];
    return t;
  }
  unsigned long long sub() const {
    unsigned long long t = 0;
    for (uint32_t i = 0; i < COUNTER_BINS; ++i) t += contacts_sub[i];
    return t;
  }
};

inline uint32_t next_pow2(uint64_t v) {
  uint32_t p = 1;
  while (p < v && p < (1u << 30)) p <<= 1;
  return p;
}
inline uint32_t ilog2(uint32_t v) {
  uint32_t l = 0;
  while ((1u << l) < v) ++l;
  return l;
}

// Bump allocator over one cudaMalloc.
struct Carver {
  size_t off = 0;
  char* base = nullptr;
  template <class T> T* take(size_t count) {
    size_t bytes = count * sizeof(T);
    size_t at = (off + 255) & ~(size_t)255;
    off = at + (bytes ? bytes : 1);
    return base ? reinterpret_cast<T*>(base + at) : nullptr;
  }
};

}  // namespace

int blobs_map_cuda(cudaError_t e) {
  if (e == cudaSuccess) return BLOBS_OK;
  if (e == cudaErrorMemoryAllocation) return BLOBS_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return BLOBS_ERR_NO_DEVICE;
  return BLOBS_ERR_CUDA;
}

struct GraphKey {
  uint32_t dt_bits;
  uint32_t cur;
  uint32_t n_steps;
  uint32_t timing;
  bool operator<(const GraphKey& o) const {
    if (dt_bits != o.dt_bits) return dt_bits < o.dt_bits;
    if (cur != o.cur) return cur < o.cur;
    if (n_steps != o.n_steps) return n_steps < o.n_steps;
    return timing < o.timing;
  }
};

// CUDA events around each kernel phase of a step (recorded into the step
// graph when timing is on), so the host can read per-phase device time.
struct TimingSet {
  struct Mark {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  void destroy() {
    for (auto& m : marks) {
      cudaEventDestroy(m.a);
      cudaEventDestroy(m.b);
    }
    marks.clear();
  }
};

struct blobs_world {
  blobs_config cfg;
  cudaStream_t stream = nullptr;
  bool loaded = false;

  uint32_t nb = 0, nc = 0, ns = 0, nj = 0, nw = 0, ncirc = 0;
  bool multiworld = false, single = false, has_springs = false, has_joints = false, rot_dynamic = false;
  bool any_dynamic = false;
  bool sorted_storage = false;  // single-sphere path: body state in cell-sorted storage (single.cu)
  int single_mode = 1;          // 0: one uniform world, 1: one world, 2: batched (single.cu)
  float v_div = 0.0f;           // sorted storage, V untracked: V[vbuf] holds the displacement of a substep of this dt
  int vbuf = 0;                 // sorted storage, V untracked: the V buffer in use
  bool pending = false;
  bool keys_valid = false;
  bool mass4r = false;          // sorted storage, every body's mass = 4 x radius
  std::vector<uint32_t> colour_offsets;  // colour k = joints [colour_offsets[k], colour_offsets[k+1]) in processing order
  std::vector<uint32_t> joint_order;     // processing position -> arena index
  float old_dt = 1.0f;
  double time = 0.0, accumulator = 0.0;
  uint32_t cur = 0;
  float2* pos[2] = {nullptr, nullptr};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  // blobs_world_snapshot: a copy of the whole device arena (every array of
  // the loaded scene, its cell tables and counters) and the host-side step
  // bookkeeping that goes with it
  struct Snapshot {
    void* mem = nullptr;
    size_t bytes = 0;
    bool valid = false;
    float old_dt = 1.0f, v_div = 0.0f;
    double time = 0.0, accumulator = 0.0;
    uint32_t cur = 0, sticky_status = 0;
    int vbuf = 0;
    bool pending = false, keys_valid = false;
  } snap;
  Counters* dcounters = nullptr;
  Counters* hcounters = nullptr;  // pinned
  WorldDev dev{};
  uint32_t sticky_status = 0;
  std::map<GraphKey, cudaGraphExec_t> graphs;
  std::map<GraphKey, uint32_t> graph_cur_after;  // storage buffer holding the state after the graph
  cudaStream_t user_stream = nullptr;  // caller's stream (NULL: the world's own)
  uint32_t timing = 0;                 // 0 off, 1 events around every phase, 2 around the contact phase only
  bool mark_open = false;              // mark_begin recorded a start event that mark_end closes
  float cell_scale = 1.0f;             // cell edge = scale x the smallest exact edge (autotuned)
  // contact recording of the eager path (adjoint recomputation)
  uint32_t* rec_list = nullptr;
  uint32_t* rec_n = nullptr;
  uint32_t* rec_max = nullptr;
  // differentiable rollout: checkpoints of the arena-order state
  struct Recording {
    bool valid = false;
    double delta = 0.0;
    uint32_t n_steps = 0, every = 0, n_seg = 0;
    float old_dt0 = 1.0f;
    bool pending0 = false;
    uint32_t substeps = 0;
    float2* ckpt = nullptr;  // (n_seg + 1) x 4 x n_bodies float2: p, po, s, v
  } rec;
  // collision event stream (physics.rs:304-311), off unless enabled
  struct HostEvent {
    uint32_t a, b;
    float va[2], vb[2];
  };
  bool events_on = false;
  void* ev_mem = nullptr;
  uint32_t ev_cap = 0;
  uint4* ev_rec = nullptr;
  float4* ev_vel = nullptr;
  uint32_t* ev_count = nullptr;
  uint32_t* ev_seq = nullptr;
  std::deque<HostEvent> ev_host;       // drained from the device, in the reference's order
  // sorted storage keeps calculated_velocity in V, double-buffered with the
  // state, when something reads it during a step (springs, events)
  bool v_tracks() const { return has_springs || events_on; }
  void attach_events() {
    dev.ev_rec = events_on ? ev_rec : nullptr;
    dev.ev_vel = events_on ? ev_vel : nullptr;
    dev.ev_count = events_on ? ev_count : nullptr;
    dev.ev_seq = events_on ? ev_seq : nullptr;
    dev.ev_cap = events_on ? ev_cap : 0u;
  }
  bool capturing = false;
  TimingSet* recording = nullptr;      // set that enqueue_substep records into
  std::map<GraphKey, TimingSet> graph_timing;
  TimingSet eager_timing;
  std::vector<TimingSet*> launched_sets;
  uint64_t kernels_launched = 0;       // kernels issued (graph nodes counted per launch)
  uint64_t enqueued = 0;               // kernels enqueued by enqueue_substep (eager or captured)
  std::map<GraphKey, uint64_t> graph_kernels;

  cudaStream_t st() const { return user_stream ? user_stream : stream; }

  ~blobs_world() { release(); }

  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    graph_cur_after.clear();
    for (auto& kv : graph_timing) kv.second.destroy();
    graph_timing.clear();
    eager_timing.destroy();
    launched_sets.clear();
  }
  // the recorded rollout (checkpoints sized for the loaded scene) is dropped
  void drop_recording() {
    if (rec.ckpt) cudaFree(rec.ckpt);
    rec = Recording();
  }
  void drop_snapshot() {
    if (snap.mem) cudaFree(snap.mem);
    snap = Snapshot();
  }
  void release() {
    drop_graphs();
    drop_recording();
    drop_snapshot();
    if (ev_mem) cudaFree(ev_mem);
    ev_mem = nullptr;
    events_on = false;
    ev_host.clear();
    if (arena) cudaFree(arena);
    arena = nullptr;
    if (hcounters) cudaFreeHost(hcounters);
    hcounters = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    loaded = false;
  }
};

namespace {

// ---------------------------------------------------------------------------
// scene validation + derived host arrays
// ---------------------------------------------------------------------------
struct HostScene {
  std::vector<float2> pos, pos_old, pend_acc, vel, vreq, col_off, snap;
  std::vector<float4> jnt_anc, jnt_coef;
  std::vector<float> rot, angvel, pend_torque, mass, inertia, gmod, bound_r, col_radius, spr_rest, spr_k, spr_c,
      circles;
  std::vector<uint8_t> bflags, col_sensor;
  std::vector<uint32_t> body_world, col_world, body_col_start, body_cols, body_spr_start, body_spr, col_parent,
      col_memb, col_filt, spr_a, spr_b, jnt_a, jnt_b;
  std::vector<WorldParam> wparam;
  std::vector<uint32_t> colour_offsets, joint_order;
  std::vector<uint32_t> jb_comp_start, jb_joint_start, jb_body_start, jb_bodies, jnt_local;
  uint32_t n_cells = 0;
  bool single = false, rot_dynamic = false, pending = false, any_dynamic = false;
};

int world_of(const uint32_t* offsets, uint32_t nw, uint32_t idx) {
  // offsets is validated to be non-decreasing; binary search
  uint32_t lo = 0, hi = nw;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) / 2;
    if (offsets[mid] <= idx) lo = mid;
    else hi = mid;
  }
  return (int)lo;
}

bool check_offsets(const uint32_t* off, uint32_t nw, uint32_t total) {
  if (!off) return nw <= 1;
  if (off[0] != 0 || off[nw] != total) return false;
  for (uint32_t w = 0; w < nw; ++w)
    if (off[w + 1] < off[w]) return false;
  return true;
}

// How a scene's joints are swept (physics.rs:424-477).  joint_order maps
// processing position -> arena index; the first jb_joint_start.back() of them
// belong to the small components, block k holding components
// [jb_comp_start[k], jb_comp_start[k+1]) and bodies
// jb_bodies[jb_body_start[k] .. jb_body_start[k+1]); jnt_local[q] holds the
// block-local slots a | b << 16 of a small component's joint; colour k of the
// large components is [colour_offsets[k], colour_offsets[k+1]).
struct JointSchedule {
  std::vector<uint32_t> joint_order, colour_offsets, jb_comp_start, jb_joint_start, jb_body_start, jb_bodies,
      jnt_local;
};

// The joint processing schedule (see JointSchedule).  The bodies a chain
// of joints links form a component, and the
// joints of one component touch no body of another, so each component can
// be swept on its own -- every iteration, its joints in arena order --
// giving each body the reference's sequence of updates (physics.rs:428-431).
// Components of at most JB_MAX_JOINTS joints become one thread each of
// k_joint_blocks (shared memory, reference order); the joints of larger
// ones are greedily coloured in arena order and swept colour by colour.
// Processing order: small components block by block, then the large
// components' joints by (colour, arena index).
int joint_schedule(uint32_t nb, uint32_t nj, const uint32_t* ja, const uint32_t* jb, JointSchedule& out) {
  std::vector<uint32_t> uf(nb);
  for (uint32_t i = 0; i < nb; ++i) uf[i] = i;
  auto find = [&](uint32_t x) {
    while (uf[x] != x) x = uf[x] = uf[uf[x]];
    return x;
  };
  for (uint32_t j = 0; j < nj; ++j) {
    const uint32_t a = ja[j], b = jb[j];
    if (a >= nb || b >= nb || a == b) return BLOBS_ERR_INVALID_ARGUMENT;
    const uint32_t ra = find(a), rb = find(b);
    if (ra != rb) uf[std::max(ra, rb)] = std::min(ra, rb);
  }
  std::vector<uint32_t> comp_joints(nj ? nb : 0, 0), comp_first(nj ? nb : 0, 0xffffffffu);
  for (uint32_t j = 0; j < nj; ++j) {
    const uint32_t r = find(ja[j]);
    if (comp_joints[r]++ == 0) comp_first[r] = j;
  }
  std::vector<uint32_t> small;  // roots of the small components, in processing order
  for (uint32_t r = 0; r < (nj ? nb : 0); ++r)
    if (comp_joints[r] && comp_joints[r] <= JB_MAX_JOINTS) small.push_back(r);
  std::sort(small.begin(), small.end(), [&](uint32_t x, uint32_t y) {
    return comp_joints[x] != comp_joints[y] ? comp_joints[x] > comp_joints[y] : comp_first[x] < comp_first[y];
  });
  // Deal the components, largest first, over the blocks in snake order, so
  // that the largest (the longest sequential sweeps) land in different blocks
  // and every block gets a similar share of the work; inside a block they stay
  // largest first.  A component of n joints has at most n + 1 bodies.
  std::vector<uint32_t> block_first(1, 0);  // component index at which each block starts (in `small`)
  if (!small.empty()) {
    uint64_t tot_j = 0;
    for (uint32_t r : small) tot_j += comp_joints[r];
    uint64_t nblk = std::max<uint64_t>({(small.size() + JB_THREADS - 1) / JB_THREADS,
                                        (tot_j * 4 + 3 * JB_JOINTS - 1) / (3 * JB_JOINTS),
                                        ((tot_j + small.size()) * 4 + 3 * JB_BODIES - 1) / (3 * JB_BODIES), 1});
    std::vector<std::vector<uint32_t>> dealt;
    while (true) {
      nblk = std::min<uint64_t>(nblk, small.size());
      dealt.assign(nblk, {});
      std::vector<uint32_t> nj_in(nblk, 0), nb_in(nblk, 0);
      bool fits = true;
      for (size_t i = 0; i < small.size() && fits; ++i) {
        const uint64_t round = i / nblk, pos = i % nblk;
        uint64_t k = (round & 1) ? nblk - 1 - pos : pos;
        const uint32_t cj = comp_joints[small[i]];
        uint64_t tries = 0;
        while (dealt[k].size() == (size_t)JB_THREADS || nj_in[k] + cj > JB_JOINTS || nb_in[k] + cj + 1 > JB_BODIES) {
          k = (k + 1) % nblk;
          if (++tries == nblk) {
            fits = false;
            break;
          }
        }
        if (!fits) break;
        dealt[k].push_back(small[i]);
        nj_in[k] += cj;
        nb_in[k] += cj + 1;
      }
      if (fits) break;
      nblk += nblk / 8 + 1;
    }
    small.clear();
    for (const auto& d : dealt) {
      small.insert(small.end(), d.begin(), d.end());
      block_first.push_back((uint32_t)small.size());
    }
  }
  std::vector<uint32_t> comp_index(nj ? nb : 0, 0xffffffffu);
  for (uint32_t c = 0; c < (uint32_t)small.size(); ++c) comp_index[small[c]] = c;
  out.jb_joint_start.assign(small.size() + 1, 0);
  for (uint32_t c = 0; c < (uint32_t)small.size(); ++c)
    out.jb_joint_start[c + 1] = out.jb_joint_start[c] + comp_joints[small[c]];
  const uint32_t n_small = small.empty() ? 0u : out.jb_joint_start.back();
  out.joint_order.assign(nj, 0);
  std::vector<uint32_t> large;  // the large components' joints, arena order
  {
    std::vector<uint32_t> fill(out.jb_joint_start.begin(), out.jb_joint_start.end() - (small.empty() ? 0 : 1));
    for (uint32_t j = 0; j < nj; ++j) {
      const uint32_t c = comp_index[find(ja[j])];
      if (c != 0xffffffffu) out.joint_order[fill[c]++] = j;
      else large.push_back(j);
    }
  }
  // the blocks' bodies, each with its block-local slot
  out.jb_comp_start.assign(block_first.begin(), block_first.end());
  out.jb_body_start.assign(1, 0);
  out.jb_bodies.clear();
  out.jnt_local.assign(nj, 0);
  {
    std::vector<int32_t> slot(nj ? nb : 0, -1);
    size_t blk = 0;
    for (uint32_t c = 0; c < (uint32_t)small.size(); ++c) {
      if (c == block_first[blk + 1]) {
        for (uint32_t i = out.jb_body_start.back(); i < (uint32_t)out.jb_bodies.size(); ++i)
          slot[out.jb_bodies[i]] = -1;
        out.jb_body_start.push_back((uint32_t)out.jb_bodies.size());
        ++blk;
      }
      const uint32_t q0 = out.jb_joint_start[c], q1 = out.jb_joint_start[c + 1];
      for (uint32_t q = q0; q < q1; ++q) {
        const uint32_t j = out.joint_order[q];
        uint32_t loc[2];
        const uint32_t ends[2] = {ja[j], jb[j]};
        for (int e2 = 0; e2 < 2; ++e2) {
          if (slot[ends[e2]] < 0) {
            slot[ends[e2]] = (int32_t)((uint32_t)out.jb_bodies.size() - out.jb_body_start.back());
            out.jb_bodies.push_back(ends[e2]);
          }
          loc[e2] = (uint32_t)slot[ends[e2]];
        }
        out.jnt_local[q] = loc[0] | (loc[1] << 16);
      }
    }
    if (!small.empty()) out.jb_body_start.push_back((uint32_t)out.jb_bodies.size());
  }
  // the large components: greedy colouring in arena order
  std::vector<uint32_t> colour(large.size(), 0);
  uint32_t n_colours = 0;
  {
    std::vector<std::vector<uint32_t>> used(large.empty() ? 0 : nb);
    for (size_t i = 0; i < large.size(); ++i) {
      const uint32_t a = ja[large[i]], b = jb[large[i]];
      uint32_t k = 0;
      while (std::find(used[a].begin(), used[a].end(), k) != used[a].end() ||
             std::find(used[b].begin(), used[b].end(), k) != used[b].end())
        ++k;
      colour[i] = k;
      used[a].push_back(k);
      used[b].push_back(k);
      n_colours = std::max(n_colours, k + 1);
    }
  }
  out.colour_offsets.assign(n_colours + 1, n_small);
  for (size_t i = 0; i < large.size(); ++i) out.colour_offsets[colour[i] + 1]++;
  for (uint32_t k = 0; k < n_colours; ++k) out.colour_offsets[k + 1] += out.colour_offsets[k] - n_small;
  {
    std::vector<uint32_t> fill(out.colour_offsets.begin(), out.colour_offsets.end() - 1);
    for (size_t i = 0; i < large.size(); ++i) out.joint_order[fill[colour[i]]++] = large[i];
  }
  return BLOBS_OK;
}

int build_host_scene(const blobs_config& cfg, float cell_scale, const blobs_scene& s, HostScene& h) {
  const uint32_t nw = s.n_worlds ? s.n_worlds : 1;
  const uint32_t nb = s.n_bodies, nc = s.n_colliders, ns = s.n_springs, nj = s.n_joints;
  if (nb && (!s.pos || !s.mass || !s.inertia)) return BLOBS_ERR_INVALID_ARGUMENT;
  if (nc && (!s.col_parent || !s.col_radius)) return BLOBS_ERR_INVALID_ARGUMENT;
  if (ns && (!s.spr_a || !s.spr_b || !s.spr_rest || !s.spr_k || !s.spr_c)) return BLOBS_ERR_INVALID_ARGUMENT;
  if (nj && (!s.jnt_a || !s.jnt_b || !s.jnt_anchor_a || !s.jnt_anchor_b || !s.jnt_distance || !s.jnt_target))
    return BLOBS_ERR_INVALID_ARGUMENT;
  if (s.n_circles && !s.circles) return BLOBS_ERR_INVALID_ARGUMENT;
  if (nw > 1) {
    if (!check_offsets(s.world_body_offsets, nw, nb) || !check_offsets(s.world_collider_offsets, nw, nc) ||
        !check_offsets(s.world_spring_offsets, nw, ns) || !check_offsets(s.world_joint_offsets, nw, nj))
      return BLOBS_ERR_INVALID_ARGUMENT;
  }
  auto bworld = [&](uint32_t b) -> uint32_t { return nw > 1 ? (uint32_t)world_of(s.world_body_offsets, nw, b) : 0u; };

  // bodies
  h.pos.resize(nb);
  h.pos_old.resize(nb);
  h.pend_acc.resize(nb);
  h.vel.resize(nb);
  h.vreq.resize(nb);
  h.rot.resize(nb);
  h.angvel.resize(nb);
  h.pend_torque.resize(nb);
  h.mass.resize(nb);
  h.inertia.resize(nb);
  h.gmod.resize(nb);
  h.bound_r.assign(nb, 0.0f);
  h.bflags.assign(nb, 0);
  h.body_world.resize(nb);
  std::vector<uint8_t> seen_dyn(nw, 0);
  for (uint32_t i = 0; i < nb; ++i) {
    h.pos[i] = v2(s.pos[2 * i], s.pos[2 * i + 1]);
    h.pos_old[i] = s.pos_old ? v2(s.pos_old[2 * i], s.pos_old[2 * i + 1]) : h.pos[i];
    h.pend_acc[i] = s.acc ? v2(s.acc[2 * i], s.acc[2 * i + 1]) : v2(0.0f, 0.0f);
    h.vel[i] = s.vel ? v2(s.vel[2 * i], s.vel[2 * i + 1]) : v2(0.0f, 0.0f);
    const bool vset = s.vreq_set && s.vreq_set[i];
    if (vset && !s.vreq) return BLOBS_ERR_INVALID_ARGUMENT;
    h.vreq[i] = vset ? v2(s.vreq[2 * i], s.vreq[2 * i + 1]) : v2(0.0f, 0.0f);
    h.rot[i] = s.rotation ? s.rotation[i] : 0.0f;
    h.angvel[i] = s.angvel ? s.angvel[i] : 0.0f;
    h.pend_torque[i] = s.torque ? s.torque[i] : 0.0f;
    h.gmod[i] = s.gravity_mod ? s.gravity_mod[i] : 1.0f;
    h.mass[i] = s.mass[i];
    h.inertia[i] = s.inertia[i];
    if (!(h.mass[i] > 0.0f) || !std::isfinite(h.mass[i])) return BLOBS_ERR_INVALID_ARGUMENT;
    const uint8_t type = s.body_type ? s.body_type[i] : (uint8_t)BLOBS_DYNAMIC;
    if (type > 3) return BLOBS_ERR_INVALID_ARGUMENT;
    const uint32_t w = bworld(i);
    h.body_world[i] = w;
    uint8_t f = 0;
    if (type == BLOBS_STATIC) {
      f |= BF_STATIC;
    } else {
      h.any_dynamic = true;
      if (!seen_dyn[w]) {
        f |= BF_FIRST_DYN;
        seen_dyn[w] = 1;
      }
    }
    if (vset) f |= BF_VREQ;
    h.bflags[i] = f;
    if (vset || h.pend_acc[i].x != 0.0f || h.pend_acc[i].y != 0.0f || h.pend_torque[i] != 0.0f) h.pending = true;
    if (h.angvel[i] != 0.0f || h.pend_torque[i] != 0.0f) h.rot_dynamic = true;
  }

  // colliders
  h.col_parent.resize(nc);
  h.col_off.resize(nc);
  h.col_radius.resize(nc);
  h.col_sensor.resize(nc);
  h.col_memb.resize(nc);
  h.col_filt.resize(nc);
  h.snap.resize(nc);
  h.col_world.resize(nc);
  std::vector<uint32_t> per_body(nb + 1, 0);
  bool single = (nc == nb);
  for (uint32_t c = 0; c < nc; ++c) {
    const uint32_t p = s.col_parent[c];
    if (p >= nb) return BLOBS_ERR_INVALID_ARGUMENT;
    const uint32_t w = nw > 1 ? (uint32_t)world_of(s.world_collider_offsets, nw, c) : 0u;
    if (w != h.body_world[p]) return BLOBS_ERR_INVALID_ARGUMENT;
    h.col_world[c] = w;
    h.col_parent[c] = p;
    h.col_off[c] = s.col_offset ? v2(s.col_offset[2 * c], s.col_offset[2 * c + 1]) : v2(0.0f, 0.0f);
    h.col_radius[c] = s.col_radius[c];
    if (!(h.col_radius[c] >= 0.0f) || !std::isfinite(h.col_radius[c])) return BLOBS_ERR_INVALID_ARGUMENT;
    h.col_sensor[c] = s.col_sensor ? (s.col_sensor[c] ? 1 : 0) : 0;
    h.col_memb[c] = s.col_memb ? s.col_memb[c] : 0xffffffffu;
    h.col_filt[c] = s.col_filt ? s.col_filt[c] : 0xffffffffu;
    if (s.col_snap) {
      h.snap[c] = v2(s.col_snap[2 * c], s.col_snap[2 * c + 1]);
    } else {
      const float sn = std::sin(h.rot[p]), cs = std::cos(h.rot[p]);
      const float2 o = h.col_off[c];
      h.snap[c] = add(v2((cs * o.x) + ((-sn) * o.y), (sn * o.x) + (cs * o.y)), h.pos[p]);
    }
    const float br = len2(h.col_off[c]) + h.col_radius[c];
    if (br > h.bound_r[p]) h.bound_r[p] = br;
    per_body[p + 1]++;
    if (p != c || h.col_off[c].x != 0.0f || h.col_off[c].y != 0.0f || h.col_sensor[c] ||
        h.col_memb[c] != 0xffffffffu || h.col_filt[c] != 0xffffffffu)
      single = false;
  }
  h.single = single;
  h.body_col_start.resize(nb + 1);
  h.body_col_start[0] = 0;
  for (uint32_t b = 0; b < nb; ++b) h.body_col_start[b + 1] = h.body_col_start[b] + per_body[b + 1];
  h.body_cols.resize(nc);
  {
    std::vector<uint32_t> fill(h.body_col_start.begin(), h.body_col_start.end() - 1);
    for (uint32_t c = 0; c < nc; ++c) h.body_cols[fill[h.col_parent[c]]++] = c;
  }

  // springs -> per-body incident list in ascending spring index
  h.spr_a.resize(ns);
  h.spr_b.resize(ns);
  h.spr_rest.resize(ns);
  h.spr_k.resize(ns);
  h.spr_c.resize(ns);
  std::vector<uint32_t> spr_count(nb + 1, 0);
  for (uint32_t i = 0; i < ns; ++i) {
    const uint32_t a = s.spr_a[i], b = s.spr_b[i];
    if (a >= nb || b >= nb || a == b) return BLOBS_ERR_INVALID_ARGUMENT;
    if (h.body_world[a] != h.body_world[b]) return BLOBS_ERR_INVALID_ARGUMENT;
    if (nw > 1 && (uint32_t)world_of(s.world_spring_offsets, nw, i) != h.body_world[a])
      return BLOBS_ERR_INVALID_ARGUMENT;
    h.spr_a[i] = a;
    h.spr_b[i] = b;
    h.spr_rest[i] = s.spr_rest[i];
    h.spr_k[i] = s.spr_k[i];
    h.spr_c[i] = s.spr_c[i];
    spr_count[a + 1]++;
    spr_count[b + 1]++;
  }
  h.body_spr_start.resize(nb + 1);
  h.body_spr_start[0] = 0;
  for (uint32_t b = 0; b < nb; ++b) h.body_spr_start[b + 1] = h.body_spr_start[b] + spr_count[b + 1];
  h.body_spr.resize(2 * (size_t)ns);
  {
    std::vector<uint32_t> fill(h.body_spr_start.begin(), h.body_spr_start.end() - 1);
    for (uint32_t i = 0; i < ns; ++i) {
      h.body_spr[fill[h.spr_a[i]]++] = (i << 1);
      h.body_spr[fill[h.spr_b[i]]++] = (i << 1) | 1u;
    }
  }

  for (uint32_t j = 0; j < nj; ++j) {
    const uint32_t a = s.jnt_a[j], b = s.jnt_b[j];
    if (a >= nb || b >= nb || a == b) return BLOBS_ERR_INVALID_ARGUMENT;
    if (h.body_world[a] != h.body_world[b]) return BLOBS_ERR_INVALID_ARGUMENT;
    if (nw > 1 && (uint32_t)world_of(s.world_joint_offsets, nw, j) != h.body_world[a])
      return BLOBS_ERR_INVALID_ARGUMENT;
  }
  {
    JointSchedule js;
    const int st = joint_schedule(nb, nj, s.jnt_a, s.jnt_b, js);
    if (st) return st;
    h.joint_order = std::move(js.joint_order);
    h.colour_offsets = std::move(js.colour_offsets);
    h.jb_comp_start = std::move(js.jb_comp_start);
    h.jb_joint_start = std::move(js.jb_joint_start);
    h.jb_body_start = std::move(js.jb_body_start);
    h.jb_bodies = std::move(js.jb_bodies);
    h.jnt_local = std::move(js.jnt_local);
  }
  h.jnt_a.resize(nj);
  h.jnt_b.resize(nj);
  h.jnt_anc.resize(nj);
  h.jnt_coef.resize(nj);
  for (uint32_t q = 0; q < nj; ++q) {
    const uint32_t j = h.joint_order[q];
    const uint32_t a = s.jnt_a[j], b = s.jnt_b[j];
    h.jnt_a[q] = a;
    h.jnt_b[q] = b;
    h.jnt_anc[q] = make_float4(s.jnt_anchor_a[2 * j], s.jnt_anchor_a[2 * j + 1], s.jnt_anchor_b[2 * j],
                               s.jnt_anchor_b[2 * j + 1]);
    // physics.rs:445-452 mass terms, IEEE f32 as the device would compute them
    const float inv_a = 1.0f / h.mass[a];
    const float ims = inv_a + (1.0f / h.mass[b]);
    h.jnt_coef[q] = make_float4(ims, inv_a / ims, s.jnt_distance[j], s.jnt_target[j]);
    if (h.bflags[a] & BF_STATIC) h.jnt_local[q] |= JL_STATIC_A;
    if (h.bflags[b] & BF_STATIC) h.jnt_local[q] |= JL_STATIC_B;
  }
  if (nj) h.rot_dynamic = true;

  h.circles.assign(s.circles, s.circles + 3 * (size_t)s.n_circles);

  // per-world toroidal grids
  h.wparam.resize(nw);
  uint64_t cell_base = 0;
  for (uint32_t w = 0; w < nw; ++w) {
    const uint32_t c0 = nw > 1 ? s.world_collider_offsets[w] : 0u;
    const uint32_t c1 = nw > 1 ? s.world_collider_offsets[w + 1] : nc;
    float rmax = 0.0f;
    float lo_x = INFINITY, lo_y = INFINITY, hi_x = -INFINITY, hi_y = -INFINITY;
    for (uint32_t c = c0; c < c1; ++c) {
      rmax = std::max(rmax, h.col_radius[c]);
      const float2 p = h.snap[c];
      if (std::isfinite(p.x) && std::isfinite(p.y)) {
        lo_x = std::min(lo_x, p.x);
        hi_x = std::max(hi_x, p.x);
        lo_y = std::min(lo_y, p.y);
        hi_y = std::max(hi_y, p.y);
      }
    }
    // The 3x3 search is exact when cs >= 2 * rmax; the 1/64 margin absorbs
    // the rounding of v / cs for coordinates up to ~1e5 cells.
    const float safe = rmax > 0.0f ? 2.0f * rmax * (1.0f + 1.0f / 64.0f) : 1.0f;
    // cell_scale >= 1 (the autotuner's choice) only enlarges cells
    const float tuned = safe * std::max(cell_scale, 1.0f);
    const float cs = cfg.cell_size > tuned ? cfg.cell_size : tuned;
    if (s.world_box) {  // bodies stay inside the walls: grid the whole box
      lo_x = std::min(lo_x, s.world_box[4 * w + 0]);
      lo_y = std::min(lo_y, s.world_box[4 * w + 1]);
      hi_x = std::max(hi_x, s.world_box[4 * w + 2]);
      hi_y = std::max(hi_y, s.world_box[4 * w + 3]);
    }
    const double ex = hi_x >= lo_x ? (double)hi_x - lo_x : 0.0, ey = hi_y >= lo_y ? (double)hi_y - lo_y : 0.0;
    uint32_t W = next_pow2(std::max<uint64_t>(4, (uint64_t)std::ceil(ex / cs) + 3));
    uint32_t H = next_pow2(std::max<uint64_t>(4, (uint64_t)std::ceil(ey / cs) + 3));
    const uint64_t cap = std::max<uint64_t>(16, 2ull * next_pow2(std::max<uint32_t>(1, c1 - c0)));
    while ((uint64_t)W * H > cap) {
      if (W >= H && W > 4) W >>= 1;
      else if (H > 4) H >>= 1;
      else break;
    }
    WorldParam& wp = h.wparam[w];
    std::memset(&wp, 0, sizeof(wp));
    wp.cell_base = (uint32_t)cell_base;
    wp.log2w = ilog2(W);
    wp.log2h = ilog2(H);
    wp.cs = cs;
    wp.inv_cs = 1.0f / cs;
    // one empty cell column / row before the extent, so the world's cells
    // are 1 .. W-2 and a 3x3 search inside it never wraps
    wp.ox = std::isfinite(lo_x) ? lo_x - cs : 0.0f;
    wp.oy = std::isfinite(lo_y) ? lo_y - cs : 0.0f;
    if (s.world_box) {
      wp.has_box = 1;
      wp.box_lo_x = s.world_box[4 * w + 0];
      wp.box_lo_y = s.world_box[4 * w + 1];
      wp.box_hi_x = s.world_box[4 * w + 2];
      wp.box_hi_y = s.world_box[4 * w + 3];
    }
    cell_base += (uint64_t)W * H;
    if (cell_base >= (1ull << 31)) return BLOBS_ERR_INVALID_ARGUMENT;
  }
  h.n_cells = (uint32_t)cell_base;

  return BLOBS_OK;
}

template <class T> cudaError_t up(T* dst, const std::vector<T>& src, cudaStream_t st) {
  if (src.empty()) return cudaSuccess;
  return cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

// Lay out (or size) every device array of the scene.
void carve(Carver& cv, WorldDev& d, float2** pos, Counters** counters, const HostScene& h, uint32_t nb, uint32_t nc,
           uint32_t ns, uint32_t nj, uint32_t nw, uint32_t ncirc, uint32_t n_cells, uint32_t n_tiles,
           bool sorted_storage) {
  const uint32_t ss = sorted_storage ? nb : 0u;
  d.sa[0] = cv.take<float4>(ss);
  d.sa[1] = cv.take<float4>(ss);
  d.sb[0] = cv.take<float4>(ss);
  d.sb[1] = cv.take<float4>(ss);
  d.sv[0] = cv.take<float2>(ss);
  d.sv[1] = cv.take<float2>(ss);
  d.cand = cv.take<float4>(ss);
  d.body_c = cv.take<float4>(ss);
  d.key = cv.take<uint32_t>(ss);
  d.ckey = cv.take<uint32_t>(ss);
  d.where = cv.take<uint32_t>(ss);
  d.defer_list = cv.take<uint32_t>(ss);
  d.defer_count = cv.take<uint32_t>(sorted_storage ? 1u : 0u);
  pos[0] = cv.take<float2>(nb);
  pos[1] = cv.take<float2>(nb);
  d.pos_old = cv.take<float2>(nb);
  d.vel = cv.take<float2>(nb);
  d.acc = cv.take<float2>(ns ? nb : 0);
  d.rot = cv.take<float>(nb);
  d.angvel = cv.take<float>(nb);
  d.mass = cv.take<float>(nb);
  d.inertia = cv.take<float>(nb);
  d.gmod = cv.take<float>(nb);
  d.bound_r = cv.take<float>(nb);
  d.bflags = cv.take<uint8_t>(nb);
  d.pend_acc = cv.take<float2>(nb);
  d.pend_torque = cv.take<float>(nb);
  d.vreq = cv.take<float2>(nb);
  d.body_world = cv.take<uint32_t>(nb);
  d.body_col_start = cv.take<uint32_t>(nb + 1);
  d.body_cols = cv.take<uint32_t>(nc);
  d.body_spr_start = cv.take<uint32_t>(nb + 1);
  d.body_spr = cv.take<uint32_t>(2 * (size_t)ns);
  d.col_parent = cv.take<uint32_t>(nc);
  d.col_off = cv.take<float2>(nc);
  d.col_radius = cv.take<float>(nc);
  d.col_memb = cv.take<uint32_t>(nc);
  d.col_filt = cv.take<uint32_t>(nc);
  d.col_sensor = cv.take<uint8_t>(nc);
  d.snap = cv.take<float2>(nc);
  d.col_world = cv.take<uint32_t>(nc);
  d.spr_a = cv.take<uint32_t>(ns);
  d.spr_b = cv.take<uint32_t>(ns);
  d.spr_rest = cv.take<float>(ns);
  d.spr_k = cv.take<float>(ns);
  d.spr_c = cv.take<float>(ns);
  d.jnt_a = cv.take<uint32_t>(nj);
  d.jnt_b = cv.take<uint32_t>(nj);
  d.jnt_anc = cv.take<float4>(nj);
  d.jnt_coef = cv.take<float4>(nj);
  d.jb_comp_start = cv.take<uint32_t>(h.jb_comp_start.size());
  d.jb_joint_start = cv.take<uint32_t>(h.jb_joint_start.size());
  d.jb_body_start = cv.take<uint32_t>(h.jb_body_start.size());
  d.jb_bodies = cv.take<uint32_t>(h.jb_bodies.size());
  d.jnt_local = cv.take<uint32_t>(h.jnt_local.size());
  d.circles = cv.take<float>(3 * (size_t)ncirc);
  d.wparam = cv.take<WorldParam>(nw);
  d.cell_count = cv.take<uint32_t>(n_cells);
  d.cell_start = cv.take<uint32_t>((size_t)n_cells + 1);
  d.rank = cv.take<uint32_t>(nc);
  d.sorted = cv.take<float4>(sorted_storage ? 0u : nc);
  d.clist = cv.take<Contact>(sorted_storage ? 0u : (size_t)nc * CL_CAP);
  d.ccount = cv.take<uint8_t>(sorted_storage ? 0u : nc);
  d.bslow = cv.take<uint8_t>(sorted_storage ? 0u : nb);
  d.tile_sums = cv.take<uint32_t>(n_tiles);
  *counters = cv.take<Counters>(1);
}

}  // namespace

// ---------------------------------------------------------------------------
// substep / step orchestration
// ---------------------------------------------------------------------------
namespace {

enum { PHASE_SCAN = 0, PHASE_SCATTER = 1, PHASE_CONTACT = 2, PHASE_JOINTS = 3, PHASE_INTEGRATE = 4, N_PHASES = 5 };

void mark_begin(blobs_world* w, int phase) {
  w->mark_open = false;
  if (!w->recording || (w->timing == 2 && phase != PHASE_CONTACT)) return;
  w->mark_open = true;
  TimingSet::Mark m{phase, nullptr, nullptr};
  cudaEventCreate(&m.a);
  cudaEventCreate(&m.b);
  if (w->capturing) cudaEventRecordWithFlags(m.a, w->st(), cudaEventRecordExternal);
  else cudaEventRecord(m.a, w->st());
  w->recording->marks.push_back(m);
}

void mark_end(blobs_world* w) {
  if (!w->recording || !w->mark_open) return;
  w->mark_open = false;
  cudaEvent_t b = w->recording->marks.back().b;
  if (w->capturing) cudaEventRecordWithFlags(b, w->st(), cudaEventRecordExternal);
  else cudaEventRecord(b, w->st());
}

void enqueue_substep(blobs_world* w, float dt, float old_dt, bool pending, bool first_in_step, bool last_in_step) {
  const WorldDev& d = w->dev;
  float2* in = w->pos[w->cur];
  float2* out = w->pos[w->cur ^ 1u];
  const bool coll = w->cfg.collisions_enabled && w->nc > 0;
  cudaStream_t st = w->st();
  const uint64_t n_colours = w->colour_offsets.empty() ? 0 : w->colour_offsets.size() - 1;
  auto joints = [&](float2* p) {
    mark_begin(w, PHASE_JOINTS);
    if (d.n_jblocks && w->cfg.joint_iterations) {
      launch_joint_blocks(d, p, dt, w->cfg.joint_iterations, st);
      w->enqueued += 1;
    }
    for (uint32_t it = 0; it < w->cfg.joint_iterations; ++it)
      for (size_t k = 0; k < n_colours; ++k) launch_joints(d, p, w->colour_offsets[k], w->colour_offsets[k + 1], dt, st);
    w->enqueued += (uint64_t)w->cfg.joint_iterations * n_colours;
    mark_end(w);
  };
  if (w->sorted_storage) {
    // the first substep of a step re-sorts the body storage into cell order;
    // the others only scatter a cell-order copy of the snapshot records
    const int cur = (int)w->cur;
    SingleArgs a;
    std::memset(&a, 0, sizeof(a));
    a.dt = dt;
    a.ratio_first = dt / old_dt;
    a.ratio_rest = dt / dt;
    a.pending = pending ? 1u : 0u;
    a.springs = w->has_springs ? 1u : 0u;
    a.rot_dynamic = w->rot_dynamic ? 1u : 0u;
    a.write_v = last_in_step ? 1u : 0u;
    a.move_v = w->v_tracks() ? 1u : 0u;
    a.v_vel = w->v_tracks() ? 1u : 0u;
    a.mass4r = w->mass4r ? 1u : 0u;
    a.rec_list = w->rec_list;
    a.rec_n = w->rec_n;
    a.rec_max = w->rec_max;
    int in = cur, out = cur ^ 1;
    if (coll) {
      if (!w->keys_valid) {
        launch_keys_single(d, d.sa[cur], w->single_mode, st);
        w->enqueued += 1;
      }
      mark_begin(w, PHASE_SCAN);
      w->enqueued += launch_scan(d, st);
      mark_end(w);
      mark_begin(w, PHASE_SCATTER);
      if (first_in_step) {
        a.a_in = d.sa[cur];
        a.b_in = d.sb[cur];
        a.v_in = d.sv[cur];
        a.a_out = d.sa[cur ^ 1];
        a.b_out = d.sb[cur ^ 1];
        a.v_out = d.sv[cur ^ 1];
        launch_permute(d, a, st);
        in = cur ^ 1;
        out = cur;
        a.cand = d.sa[in];
        a.own_cell = d.ckey;
      } else {
        launch_scatter_cand(d, d.sa[cur], d.cand, st);
        a.cand = d.cand;
        a.own_cell = d.key;
      }
      mark_end(w);
      a.contacts = 1u;
      a.do_keys = 1u;
      w->enqueued += 2;  // permute or scatter, step
      w->keys_valid = true;
    } else {
      w->enqueued += 1;
      w->keys_valid = false;
    }
    a.a_in = d.sa[in];
    a.b_in = d.sb[in];
    a.v_in = d.sv[w->v_tracks() ? in : w->vbuf];
    a.a_out = d.sa[out];
    a.b_out = d.sb[out];
    a.v_out = d.sv[w->v_tracks() ? out : w->vbuf];
    mark_begin(w, coll ? PHASE_CONTACT : PHASE_INTEGRATE);
    launch_step_single(d, a, w->single_mode, st);
    if (coll) {
      // bodies with many candidates, deferred by the step kernel, a warp each
      launch_step_deferred(d, a, w->single_mode, st);
      w->enqueued += 1;
    }
    mark_end(w);
    if (coll && d.ev_rec) {
      launch_ev_tick(d, st);
      w->enqueued += 1;
    }
    w->cur = (uint32_t)out;
    if (!w->v_tracks() && last_in_step) w->v_div = dt;
    return;
  }
  if (coll && !w->keys_valid) {
    launch_keys(d, w->multiworld, st);
    w->enqueued += 1;
  }
  if (coll) {
    mark_begin(w, PHASE_SCAN);
    w->enqueued += launch_scan(d, st);
    mark_end(w);
  }
  if (coll || w->has_springs) {
    mark_begin(w, PHASE_SCATTER);
    launch_scatter_forces(d, in, w->multiworld, coll, w->has_springs, pending, st);
    mark_end(w);
    w->enqueued += 1;
  }
  if (coll) {
    // events read the start-of-substep velocities, which the fused
    // integration would overwrite in place
    const bool fuse = !w->has_joints && !w->events_on;
    mark_begin(w, PHASE_CONTACT);
    w->enqueued += launch_contacts(d, in, out, w->multiworld, w->single, w->has_springs, pending, fuse, dt, old_dt,
                                   true, w->rot_dynamic, st);
    mark_end(w);
    if (d.ev_rec) {
      launch_ev_tick(d, st);
      w->enqueued += 1;
    }
    if (!fuse) {
      joints(out);
      mark_begin(w, PHASE_INTEGRATE);
      launch_integrate(d, out, out, w->multiworld, w->single, w->has_springs, pending, dt, old_dt, true,
                       w->rot_dynamic, st);
      mark_end(w);
      w->enqueued += 1;
    }
    w->keys_valid = true;
  } else {
    if (w->has_joints) joints(in);
    mark_begin(w, PHASE_INTEGRATE);
    launch_integrate(d, in, out, w->multiworld, w->single, w->has_springs, pending, dt, old_dt, false,
                     w->rot_dynamic, st);
    mark_end(w);
    w->enqueued += 1;
    w->keys_valid = false;
  }
  w->cur ^= 1u;
}

// One reference `integrate(substeps, delta)` (physics.rs:397-422) enqueued
// eagerly, honouring pending requests and the old_dt ratio.
void enqueue_integrate(blobs_world* w, float delta) {
  const float step_delta = delta / (float)w->cfg.substeps;
  for (uint32_t s = 0; s < w->cfg.substeps; ++s) {
    enqueue_substep(w, step_delta, w->old_dt, w->pending, s == 0, s + 1 == w->cfg.substeps);
    w->pending = false;
    if (w->any_dynamic) w->old_dt = step_delta;
  }
}

uint32_t f2bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

// `n_steps` steady-state steps (no pending request, old_dt == step delta)
// from one cached CUDA graph.
int launch_steady(blobs_world* w, float delta, uint32_t n_steps) {
  const float step_delta = delta / (float)w->cfg.substeps;
  const bool coll = w->cfg.collisions_enabled && w->nc > 0;
  if (coll && !w->keys_valid) {
    if (w->sorted_storage) launch_keys_single(w->dev, w->dev.sa[w->cur], w->single_mode, w->st());
    else launch_keys(w->dev, w->multiworld, w->st());
    w->keys_valid = true;
  }
  // the buffers baked into a graph depend on where the state is now
  GraphKey key{f2bits(delta), w->cur | ((uint32_t)w->vbuf << 1), n_steps, w->timing};
  auto it = w->graphs.find(key);
  const uint32_t cur0 = w->cur;
  if (it == w->graphs.end()) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(w->st(), cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return blobs_map_cuda(e);
    w->capturing = true;
    w->recording = w->timing ? &w->graph_timing[key] : nullptr;
    const uint64_t before = w->enqueued;
    for (uint32_t n = 0; n < n_steps; ++n)
      for (uint32_t s = 0; s < w->cfg.substeps; ++s)
        enqueue_substep(w, step_delta, step_delta, false, s == 0, s + 1 == w->cfg.substeps);
    w->capturing = false;
    w->recording = nullptr;
    w->graph_kernels[key] = w->enqueued - before;
    w->graph_cur_after[key] = w->cur;
    w->enqueued = before;
    e = cudaStreamEndCapture(w->st(), &g);
    if (e != cudaSuccess) {
      w->cur = cur0;  // nothing ran
      return blobs_map_cuda(e);
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return blobs_map_cuda(e);
    it = w->graphs.emplace(key, ge).first;
    w->cur = cur0;  // capture did not execute anything
  }
  cudaError_t e = cudaGraphLaunch(it->second, w->st());
  if (e != cudaSuccess) return blobs_map_cuda(e);
  w->kernels_launched += w->graph_kernels[key];
  if (w->timing) {
    TimingSet* ts = &w->graph_timing[key];
    if (std::find(w->launched_sets.begin(), w->launched_sets.end(), ts) == w->launched_sets.end())
      w->launched_sets.push_back(ts);
  }
  w->cur = w->graph_cur_after[key];
  if (w->sorted_storage && !w->v_tracks()) w->v_div = step_delta;
  w->keys_valid = coll;
  return BLOBS_OK;
}

int run_steps(blobs_world* w, double delta, uint32_t n_steps) {
  if (!w->loaded) return BLOBS_ERR_STATE;
  if (!(delta > 0.0) || !std::isfinite(delta)) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  const float df = (float)delta;
  const float step_delta = df / (float)w->cfg.substeps;
  uint32_t done = 0;
  // irregular first step: eager
  while (done < n_steps && (w->pending || (w->any_dynamic && f2bits(w->old_dt) != f2bits(step_delta)))) {
    if (w->timing) {
      w->recording = &w->eager_timing;
      if (std::find(w->launched_sets.begin(), w->launched_sets.end(), w->recording) == w->launched_sets.end())
        w->launched_sets.push_back(w->recording);
    }
    const uint64_t before = w->enqueued;
    enqueue_integrate(w, df);
    w->kernels_launched += w->enqueued - before;
    w->recording = nullptr;
    w->time += delta;
    ++done;
  }
  if (done < n_steps) {
    int st = launch_steady(w, df, n_steps - done);
    if (st) return st;
    w->time += delta * (double)(n_steps - done);
  }
  e = cudaGetLastError();
  return blobs_map_cuda(e);
}

// Arena-order state (p, po, s, v) of a single-sphere world into four
// n-body float2 slices (v only holds velocities in worlds with springs).
void gather_state(blobs_world* w, float2* p, float2* po, float2* sn, float2* v) {
  const int c = (int)w->cur;
  launch_gather_single(w->dev, w->dev.sa[c], w->dev.sb[c], w->dev.sv[w->v_tracks() ? c : w->vbuf], p, po,
                       w->v_tracks() ? v : nullptr, sn, 0.0f, w->st());
}

void restore_state(blobs_world* w, const float2* p, const float2* po, const float2* sn, const float2* v) {
  const int c = (int)w->cur;
  launch_write_single(w->dev, w->dev.sa[c], w->dev.sb[c], w->dev.sv[w->v_tracks() ? c : w->vbuf], p, po,
                      w->v_tracks() ? v : nullptr, sn, w->st());
  // the snapshots changed: the next substep recounts the cells from zero
  cudaMemsetAsync(w->dev.cell_count, 0, sizeof(uint32_t) * (size_t)w->dev.n_cells, w->st());
  w->keys_valid = false;
  w->v_div = 0.0f;
}

int read_status(blobs_world* w) {
  cudaError_t e = cudaMemcpyAsync(w->hcounters, w->dev.contacts_total, sizeof(Counters), cudaMemcpyDeviceToHost,
                                  w->st());
  if (e == cudaSuccess) e = cudaStreamSynchronize(w->st());
  if (e != cudaSuccess) return blobs_map_cuda(e);
  w->sticky_status |= w->hcounters->status;
  if (w->sticky_status & ST_NAN) return BLOBS_ERR_NAN;
  if (w->sticky_status & ST_TIMEOUT) return BLOBS_ERR_TIMEOUT;
  if (w->sticky_status & ST_BAD_INDEX) return BLOBS_ERR_INVALID_ARGUMENT;
  return BLOBS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// internal API shared with the other translation units
// ---------------------------------------------------------------------------
const WorldDev* blobs_world_dev(blobs_world* w) { return w && w->loaded ? &w->dev : nullptr; }
cudaStream_t blobs_world_stream(blobs_world* w) { return w ? w->st() : nullptr; }
float2* blobs_world_pos(blobs_world* w) { return w && w->loaded ? w->pos[w->cur] : nullptr; }

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int blobs_abi_version(void) { return BLOBS_ABI_VERSION; }

void blobs_config_default(blobs_config* cfg) {
  if (!cfg) return;
  cfg->gravity[0] = 0.0f;
  cfg->gravity[1] = 0.0f;
  cfg->substeps = 8;
  cfg->joint_iterations = 4;
  cfg->collisions_enabled = 1;
  cfg->cell_size = 0.0f;
  cfg->device = 0;
}

const char* blobs_status_string(int status) {
  switch (status) {
    case BLOBS_OK: return "ok";
    case BLOBS_ERR_INVALID_HANDLE: return "invalid handle";
    case BLOBS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case BLOBS_ERR_OVERFLOW: return "capacity overflow";
    case BLOBS_ERR_NAN: return "NaN in contact normal or rotation";
    case BLOBS_ERR_CUDA: return "CUDA runtime error";
    case BLOBS_ERR_TIMEOUT: return "device wait timed out";
    case BLOBS_ERR_NO_DEVICE: return "no usable CUDA device";
    case BLOBS_ERR_OUT_OF_MEMORY: return "device out of memory";
    case BLOBS_ERR_STATE: return "invalid state for this call";
    default: return "unknown status";
  }
}

int blobs_world_create(const blobs_config* cfg, blobs_world** out) {
  if (!out) return BLOBS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  blobs_config c;
  if (cfg) c = *cfg;
  else blobs_config_default(&c);
  if (c.substeps == 0) return BLOBS_ERR_INVALID_ARGUMENT;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return BLOBS_ERR_NO_DEVICE;
  if (c.device < 0 || c.device >= count) return BLOBS_ERR_INVALID_ARGUMENT;
  e = cudaSetDevice(c.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  blobs_world* w = new blobs_world();
  w->cfg = c;
  e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&w->hcounters), sizeof(Counters));
  if (e != cudaSuccess) {
    delete w;
    return blobs_map_cuda(e);
  }
  *out = w;
  return BLOBS_OK;
}

int blobs_world_destroy(blobs_world* w) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  cudaSetDevice(w->cfg.device);
  if (w->stream) cudaStreamSynchronize(w->stream);
  delete w;
  return BLOBS_OK;
}

int blobs_world_set_config(blobs_world* w, const blobs_config* cfg) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!cfg || cfg->substeps == 0 || cfg->device != w->cfg.device) return BLOBS_ERR_INVALID_ARGUMENT;
  const bool gravity_changed = cfg->gravity[0] != w->cfg.gravity[0] || cfg->gravity[1] != w->cfg.gravity[1];
  const bool cs_changed = cfg->cell_size != w->cfg.cell_size;
  w->cfg = *cfg;
  w->dev.gravity = v2(cfg->gravity[0], cfg->gravity[1]);
  w->drop_graphs();
  (void)gravity_changed;
  (void)cs_changed;
  return BLOBS_OK;
}

int blobs_world_load(blobs_world* w, const blobs_scene* scene, float old_dt) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!scene) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  HostScene h;
  int st = build_host_scene(w->cfg, w->cell_scale, *scene, h);
  if (st) return st;
  cudaStreamSynchronize(w->st());
  w->drop_graphs();
  w->drop_recording();
  w->drop_snapshot();
  if (w->arena) cudaFree(w->arena);
  w->arena = nullptr;
  w->arena_bytes = 0;
  w->loaded = false;

  const uint32_t nb = scene->n_bodies, nc = scene->n_colliders, ns = scene->n_springs, nj = scene->n_joints;
  const uint32_t nw = scene->n_worlds ? scene->n_worlds : 1, ncirc = scene->n_circles;
  const uint32_t n_tiles = (h.n_cells + SCAN_TILE - 1) / SCAN_TILE;
  WorldDev d{};
  Counters* counters = nullptr;
  Carver sizer;
  const bool sorted_storage = h.single && nj == 0;
  // a uniform single-sphere world needs no per-body constant record
  bool mass4r = sorted_storage;  // rigid_body.rs:96-128 with one collider, no override: m = 4 r
  for (uint32_t i = 0; i < nb && mass4r; ++i) mass4r = h.mass[i] == h.col_radius[i] * 4.0f;
  w->mass4r = mass4r;
  bool uniform = sorted_storage && nw == 1;
  uint32_t first_dyn = 0xffffffffu;
  for (uint32_t i = 0; i < nb && uniform; ++i) {
    if (h.bflags[i] & BF_STATIC) uniform = false;
    if (h.gmod[i] != h.gmod[0] || std::isnan(h.gmod[i])) uniform = false;
    if (!(h.mass[i] == h.col_radius[i] * 4.0f) || !(h.bound_r[i] == h.col_radius[i])) uniform = false;
    if ((h.bflags[i] & BF_FIRST_DYN) && first_dyn == 0xffffffffu) first_dyn = i;
  }
  if (!h.wparam.empty()) {
    h.wparam[0].first_dyn = first_dyn;
    h.wparam[0].uniform_gmod = nb ? h.gmod[0] : 1.0f;
  }
  carve(sizer, d, w->pos, &counters, h, nb, nc, ns, nj, nw, ncirc, h.n_cells, n_tiles, sorted_storage);
  e = cudaMalloc(&w->arena, sizer.off + 256);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  w->arena_bytes = sizer.off + 256;
  Carver cv;
  cv.base = static_cast<char*>(w->arena);
  carve(cv, d, w->pos, &counters, h, nb, nc, ns, nj, nw, ncirc, h.n_cells, n_tiles, sorted_storage);
  d.n_bodies = nb;
  d.n_cols = nc;
  d.n_springs = ns;
  d.n_joints = nj;
  d.n_worlds = nw;
  d.n_circles = ncirc;
  d.n_cells = h.n_cells;
  d.n_tiles = n_tiles;
  d.n_jblocks = h.jb_comp_start.empty() ? 0u : (uint32_t)h.jb_comp_start.size() - 1u;
  d.gravity = v2(w->cfg.gravity[0], w->cfg.gravity[1]);
  d.contacts_total = counters->contacts_total;
  d.pushouts_total = counters->pushouts_total;
  d.contacts_sub = counters->contacts_sub;
  d.defer_total = counters->defer_total;
  d.defer_sub = counters->defer_sub;
  d.status = &counters->status;
  w->dcounters = counters;

  cudaStream_t s = w->stream;
  e = cudaSuccess;
#define UP(dst, src) \
  if (e == cudaSuccess) e = up(dst, src, s)
  UP(w->pos[0], h.pos);
  UP(d.pos_old, h.pos_old);
  UP(d.vel, h.vel);
  UP(d.rot, h.rot);
  UP(d.angvel, h.angvel);
  UP(d.mass, h.mass);
  UP(d.inertia, h.inertia);
  UP(d.gmod, h.gmod);
  UP(d.bound_r, h.bound_r);
  UP(d.bflags, h.bflags);
  UP(d.pend_acc, h.pend_acc);
  UP(d.pend_torque, h.pend_torque);
  UP(d.vreq, h.vreq);
  UP(d.body_world, h.body_world);
  UP(d.body_col_start, h.body_col_start);
  UP(d.body_cols, h.body_cols);
  UP(d.body_spr_start, h.body_spr_start);
  UP(d.body_spr, h.body_spr);
  UP(d.col_parent, h.col_parent);
  UP(d.col_off, h.col_off);
  UP(d.col_radius, h.col_radius);
  UP(d.col_memb, h.col_memb);
  UP(d.col_filt, h.col_filt);
  UP(d.col_sensor, h.col_sensor);
  UP(d.snap, h.snap);
  UP(d.col_world, h.col_world);
  UP(d.spr_a, h.spr_a);
  UP(d.spr_b, h.spr_b);
  UP(d.spr_rest, h.spr_rest);
  UP(d.spr_k, h.spr_k);
  UP(d.spr_c, h.spr_c);
  UP(d.jnt_a, h.jnt_a);
  UP(d.jnt_b, h.jnt_b);
  UP(d.jnt_anc, h.jnt_anc);
  UP(d.jnt_coef, h.jnt_coef);
  UP(d.jb_comp_start, h.jb_comp_start);
  UP(d.jb_joint_start, h.jb_joint_start);
  UP(d.jb_body_start, h.jb_body_start);
  UP(d.jb_bodies, h.jb_bodies);
  UP(d.jnt_local, h.jnt_local);
  UP(d.circles, h.circles);
  UP(d.wparam, h.wparam);
#undef UP
  std::vector<float4> sa, sb, sc;
  std::vector<uint32_t> ident;
  if (sorted_storage) {
    // storage order = arena order until the first substep sorts it
    sa.resize(nb);
    sb.resize(nb);
    sc.resize(nb);
    ident.resize(nb);
    for (uint32_t i = 0; i < nb; ++i) {
      uint32_t idbits = i;
      float idf;
      std::memcpy(&idf, &idbits, 4);
      sa[i] = make_float4(h.snap[i].x, h.snap[i].y, h.col_radius[i], idf);
      sb[i] = make_float4(h.pos[i].x, h.pos[i].y, h.pos_old[i].x, h.pos_old[i].y);
      const uint32_t fw = (uint32_t)h.bflags[i] | (h.body_world[i] << 8);
      float fwf;
      std::memcpy(&fwf, &fw, 4);
      sc[i] = make_float4(h.mass[i], h.gmod[i], h.bound_r[i], fwf);
      ident[i] = i;
    }
    if (nw >= (1u << 24)) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) e = up(d.sa[0], sa, s);
    if (e == cudaSuccess) e = up(d.sb[0], sb, s);
    if (e == cudaSuccess) e = up(d.sv[0], h.vel, s);
    if (e == cudaSuccess) e = up(d.body_c, sc, s);
    if (e == cudaSuccess) e = up(d.where, ident, s);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(d.cell_count, 0, sizeof(uint32_t) * (size_t)h.n_cells, s);
  if (e == cudaSuccess && !sorted_storage) e = cudaMemsetAsync(d.bslow, 0, nb, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, sizeof(Counters), s);
  if (e == cudaSuccess && sorted_storage) e = cudaMemsetAsync(d.defer_count, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) {
    cudaFree(w->arena);
    w->arena = nullptr;
    return blobs_map_cuda(e);
  }
  w->dev = d;
  w->attach_events();
  if (w->events_on) {
    // a reloaded world starts a new event stream
    w->ev_host.clear();
    cudaMemsetAsync(w->ev_count, 0, 2 * sizeof(uint32_t), s);
  }
  w->nb = nb;
  w->nc = nc;
  w->ns = ns;
  w->nj = nj;
  w->nw = nw;
  w->ncirc = ncirc;
  w->multiworld = nw > 1;
  w->single = h.single;
  w->sorted_storage = sorted_storage;
  w->single_mode = nw > 1 ? 2 : (uniform ? 0 : 1);
  w->v_div = 0.0f;
  w->vbuf = 0;
  w->has_springs = ns > 0;
  w->has_joints = nj > 0;
  w->rot_dynamic = h.rot_dynamic;
  w->any_dynamic = h.any_dynamic;
  w->pending = h.pending;
  w->keys_valid = false;
  w->colour_offsets = h.colour_offsets;
  w->joint_order = h.joint_order;
  w->old_dt = old_dt;
  w->time = 0.0;
  w->accumulator = 0.0;
  w->cur = 0;
  w->sticky_status = 0;
  w->loaded = true;
  e = cudaStreamSynchronize(s);  // host vectors die at return
  return blobs_map_cuda(e);
}

int blobs_world_step(blobs_world* w, double delta) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  return run_steps(w, delta, 1);
}

int blobs_world_rollout(blobs_world* w, double delta, uint32_t n_steps) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (n_steps == 0) return BLOBS_OK;
  return run_steps(w, delta, n_steps);
}

int blobs_world_fixed_step(blobs_world* w, double frame_time) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  // physics.rs:84-99
  w->accumulator += frame_time;
  const double delta = 1.0 / 60.0;
  int max_steps = 3;
  while (w->accumulator >= delta && max_steps > 0) {
    int st = run_steps(w, delta, 1);
    if (st) return st;
    w->accumulator -= delta;
    max_steps -= 1;
  }
  return BLOBS_OK;
}

int blobs_world_sync(blobs_world* w) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_OK;
  cudaSetDevice(w->cfg.device);
  return read_status(w);
}

int blobs_world_read_bodies(blobs_world* w, float* pos, float* pos_old, float* vel, float* rotation, float* angvel) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  cudaSetDevice(w->cfg.device);
  const size_t n = w->nb;
  cudaError_t e = cudaSuccess;
  cudaStream_t s = w->st();
  if (w->sorted_storage) {
    // storage order -> arena order into the staging arrays, then copy out
    const int c = (int)w->cur;
    launch_gather_single(w->dev, w->dev.sa[c], w->dev.sb[c], w->dev.sv[w->v_tracks() ? c : w->vbuf],
                         pos ? w->pos[0] : nullptr, pos_old ? w->dev.pos_old : nullptr, vel ? w->dev.vel : nullptr,
                         nullptr, w->v_div, s);
    e = cudaGetLastError();
    if (e == cudaSuccess && pos && n) e = cudaMemcpyAsync(pos, w->pos[0], n * 8, cudaMemcpyDeviceToHost, s);
  } else if (pos && n) {
    e = cudaMemcpyAsync(pos, w->pos[w->cur], n * 8, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess && pos_old && n) e = cudaMemcpyAsync(pos_old, w->dev.pos_old, n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && vel && n) e = cudaMemcpyAsync(vel, w->dev.vel, n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && rotation && n) e = cudaMemcpyAsync(rotation, w->dev.rot, n * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && angvel && n) e = cudaMemcpyAsync(angvel, w->dev.angvel, n * 4, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  return read_status(w);
}

int blobs_world_read_snapshots(blobs_world* w, float* xy) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  if (!xy) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaSetDevice(w->cfg.device);
  cudaError_t e = cudaSuccess;
  if (w->sorted_storage) {
    const int c = (int)w->cur;
    launch_gather_single(w->dev, w->dev.sa[c], w->dev.sb[c], w->dev.sv[0], nullptr, nullptr, nullptr, w->dev.snap,
                         0.0f, w->st());
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && w->nc) e = cudaMemcpyAsync(xy, w->dev.snap, (size_t)w->nc * 8, cudaMemcpyDeviceToHost, w->st());
  if (e != cudaSuccess) return blobs_map_cuda(e);
  return read_status(w);
}

int blobs_world_contact_count(blobs_world* w, uint64_t* total, uint64_t* last_substep) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  cudaSetDevice(w->cfg.device);
  int st = read_status(w);
  if (total) *total = w->hcounters->contacts();
  if (last_substep) *last_substep = w->hcounters->sub();
  return st;
}

int blobs_world_pushout_count(blobs_world* w, uint64_t* total) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  cudaSetDevice(w->cfg.device);
  int st = read_status(w);
  if (total) *total = w->hcounters->pushouts();
  return st;
}

int blobs_world_deferred_count(blobs_world* w, uint64_t* total, uint64_t* last_substep) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  cudaSetDevice(w->cfg.device);
  int st = read_status(w);
  if (total) *total = w->hcounters->deferred();
  if (last_substep) *last_substep = w->hcounters->deferred_sub();
  return st;
}

int blobs_world_time(blobs_world* w, double* time, double* accumulator) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (time) *time = w->time;
  if (accumulator) *accumulator = w->accumulator;
  return BLOBS_OK;
}

int blobs_joint_schedule(uint32_t n_bodies, uint32_t n_joints, const uint32_t* jnt_a, const uint32_t* jnt_b,
                         uint32_t* order, uint32_t* block_joint_start, uint32_t* n_blocks, uint32_t* colour_start,
                         uint32_t* n_colours) {
  if (n_joints && (!jnt_a || !jnt_b)) return BLOBS_ERR_INVALID_ARGUMENT;
  JointSchedule js;
  const int st = joint_schedule(n_bodies, n_joints, jnt_a, jnt_b, js);
  if (st) return st;
  const uint32_t nblk = js.jb_comp_start.empty() ? 0u : (uint32_t)js.jb_comp_start.size() - 1u;
  const uint32_t ncol = js.colour_offsets.empty() ? 0u : (uint32_t)js.colour_offsets.size() - 1u;
  if (order && n_joints) std::memcpy(order, js.joint_order.data(), sizeof(uint32_t) * n_joints);
  if (block_joint_start)
    for (uint32_t k = 0; k <= nblk; ++k) block_joint_start[k] = js.jb_joint_start[js.jb_comp_start[k]];
  if (n_blocks) *n_blocks = nblk;
  if (colour_start)
    for (uint32_t k = 0; k <= ncol; ++k) colour_start[k] = js.colour_offsets[k];
  if (n_colours) *n_colours = ncol;
  return BLOBS_OK;
}

int blobs_world_snapshot(blobs_world* w) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  if (w->snap.bytes != w->arena_bytes) {
    w->drop_snapshot();
    e = cudaMalloc(&w->snap.mem, w->arena_bytes);
    if (e != cudaSuccess) {
      w->snap = blobs_world::Snapshot();
      return blobs_map_cuda(e);
    }
    w->snap.bytes = w->arena_bytes;
  }
  e = cudaMemcpyAsync(w->snap.mem, w->arena, w->arena_bytes, cudaMemcpyDeviceToDevice, w->st());
  if (e != cudaSuccess) return blobs_map_cuda(e);
  w->snap.valid = true;
  w->snap.old_dt = w->old_dt;
  w->snap.v_div = w->v_div;
  w->snap.time = w->time;
  w->snap.accumulator = w->accumulator;
  w->snap.cur = w->cur;
  w->snap.sticky_status = w->sticky_status;
  w->snap.vbuf = w->vbuf;
  w->snap.pending = w->pending;
  w->snap.keys_valid = w->keys_valid;
  return BLOBS_OK;
}

int blobs_world_restore(blobs_world* w) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded || !w->snap.valid || w->snap.bytes != w->arena_bytes) return BLOBS_ERR_STATE;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  e = cudaMemcpyAsync(w->arena, w->snap.mem, w->arena_bytes, cudaMemcpyDeviceToDevice, w->st());
  if (e != cudaSuccess) return blobs_map_cuda(e);
  w->old_dt = w->snap.old_dt;
  w->v_div = w->snap.v_div;
  w->time = w->snap.time;
  w->accumulator = w->snap.accumulator;
  w->cur = w->snap.cur;
  w->sticky_status = w->snap.sticky_status;
  w->vbuf = w->snap.vbuf;
  w->pending = w->snap.pending;
  w->keys_valid = w->snap.keys_valid;
  w->drop_recording();  // a recorded rollout belongs to the trajectory it recorded
  return BLOBS_OK;
}

int blobs_world_joint_order(blobs_world* w, uint32_t* order, uint32_t* n_colours) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  if (order && !w->joint_order.empty())
    std::memcpy(order, w->joint_order.data(), w->joint_order.size() * sizeof(uint32_t));
  if (n_colours) *n_colours = w->colour_offsets.empty() ? 0u : (uint32_t)(w->colour_offsets.size() - 1);
  return BLOBS_OK;
}

int blobs_world_set_stream(blobs_world* w, void* stream) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  // the legacy / per-thread default streams cannot be captured into graphs
  if (stream == (void*)cudaStreamLegacy || stream == (void*)cudaStreamPerThread) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaSetDevice(w->cfg.device);
  cudaError_t e = cudaStreamSynchronize(w->st());
  w->user_stream = static_cast<cudaStream_t>(stream);
  return blobs_map_cuda(e);
}

int blobs_world_write_bodies(blobs_world* w, const float* pos, const float* pos_old, const float* vel,
                             const float* rotation, const float* angvel) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  cudaSetDevice(w->cfg.device);
  const size_t n = w->nb;
  cudaStream_t s = w->st();
  cudaError_t e = cudaSuccess;
  float2* pos_dst = w->sorted_storage ? w->pos[0] : w->pos[w->cur];
  if (pos && n) e = cudaMemcpyAsync(pos_dst, pos, n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && pos_old && n) e = cudaMemcpyAsync(w->dev.pos_old, pos_old, n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && vel && n) e = cudaMemcpyAsync(w->dev.vel, vel, n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && w->sorted_storage && n) {
    // arena order staging -> storage order
    const int c = (int)w->cur;
    launch_write_single(w->dev, w->dev.sa[c], w->dev.sb[c], w->dev.sv[w->v_tracks() ? c : w->vbuf],
                        pos ? w->pos[0] : nullptr, pos_old ? w->dev.pos_old : nullptr, vel ? w->dev.vel : nullptr,
                        nullptr, s);
    if (vel) w->v_div = 0.0f;  // every V entry is now a velocity
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && rotation && n) e = cudaMemcpyAsync(w->dev.rot, rotation, n * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && angvel && n) {
    e = cudaMemcpyAsync(w->dev.angvel, angvel, n * 4, cudaMemcpyHostToDevice, s);
    if (!w->rot_dynamic) {  // a non-zero angular velocity needs the rotation update
      for (size_t i = 0; i < n && !w->rot_dynamic; ++i) w->rot_dynamic = angvel[i] != 0.0f;
      if (w->rot_dynamic) w->drop_graphs();
    }
  }
  return blobs_map_cuda(e);
}

int blobs_world_emit_pairs(blobs_world* w, int contacts_only, uint32_t* pairs, uint64_t cap, uint64_t* n_pairs) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  if (!n_pairs || (cap && !pairs)) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaSetDevice(w->cfg.device);
  cudaStream_t s = w->st();
  *n_pairs = 0;
  if (w->nc == 0) return read_status(w);
  // rebuild the cell ranges from the current snapshots; the next substep
  // recomputes its ranks (the scan consumed the counts)
  WorldDev dv = w->dev;
  if (w->sorted_storage) {
    const int c = (int)w->cur;
    if (!w->keys_valid) launch_keys_single(w->dev, w->dev.sa[c], w->single_mode, s);
    launch_scan(w->dev, s);
    SingleArgs a;
    std::memset(&a, 0, sizeof(a));
    a.a_in = w->dev.sa[c];
    a.b_in = w->dev.sb[c];
    // V moves with the records; without springs it lives in its own buffer
    const int vi = w->v_tracks() ? c : w->vbuf;
    a.v_in = w->dev.sv[vi];
    a.a_out = w->dev.sa[c ^ 1];
    a.b_out = w->dev.sb[c ^ 1];
    a.v_out = w->dev.sv[vi ^ 1];
    a.move_v = 1u;
    launch_permute(w->dev, a, s);
    w->cur ^= 1u;  // the permuted storage becomes current
    if (!w->v_tracks()) w->vbuf ^= 1;
    dv.sorted = w->dev.sa[w->cur];
  } else {
    if (!w->keys_valid) launch_keys(w->dev, w->multiworld, s);
    launch_scan(w->dev, s);
    launch_scatter_forces(w->dev, w->pos[w->cur], w->multiworld, true, false, false, s);
  }
  w->keys_valid = false;
  uint32_t* dpairs = nullptr;
  unsigned long long* dcount = nullptr;
  cudaError_t e = cudaMallocAsync(&dcount, sizeof(unsigned long long), s);
  if (e == cudaSuccess && cap) e = cudaMallocAsync(&dpairs, 2 * sizeof(uint32_t) * cap, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) {
    launch_emit_pairs(dv, w->multiworld, contacts_only ? 1u : 0u, dpairs, cap, dcount, s);
    e = cudaGetLastError();
  }
  unsigned long long total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, dcount, sizeof(total), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && cap)
    e = cudaMemcpyAsync(pairs, dpairs, 2 * sizeof(uint32_t) * (total < cap ? total : cap), cudaMemcpyDeviceToHost, s);
  if (dpairs) cudaFreeAsync(dpairs, s);
  if (dcount) cudaFreeAsync(dcount, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  *n_pairs = total;
  int st = read_status(w);
  if (st) return st;
  return total > cap ? BLOBS_ERR_OVERFLOW : BLOBS_OK;
}

int blobs_world_grid(blobs_world* w, uint32_t world, float* cell_size, float* inv_cell_size, float* origin,
                     uint32_t* log2_width, uint32_t* log2_height) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  if (world >= w->nw) return BLOBS_ERR_INVALID_ARGUMENT;
  WorldParam wp;
  cudaSetDevice(w->cfg.device);
  cudaError_t e = cudaMemcpy(&wp, w->dev.wparam + world, sizeof(wp), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  if (cell_size) *cell_size = wp.cs;
  if (inv_cell_size) *inv_cell_size = wp.inv_cs;
  if (origin) {
    origin[0] = wp.ox;
    origin[1] = wp.oy;
  }
  if (log2_width) *log2_width = wp.log2w;
  if (log2_height) *log2_height = wp.log2h;
  return BLOBS_OK;
}

int blobs_world_rollout_record(blobs_world* w, double delta, uint32_t n_steps, uint32_t checkpoint_every) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded) return BLOBS_ERR_STATE;
  if (!w->sorted_storage || w->ncirc || n_steps == 0 || checkpoint_every == 0) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaSetDevice(w->cfg.device);
  auto& r = w->rec;
  if (r.ckpt) cudaFree(r.ckpt);
  r = blobs_world::Recording();
  const uint32_t n_seg = (n_steps + checkpoint_every - 1) / checkpoint_every;
  const size_t nb = w->nb;
  cudaError_t e = cudaMalloc(&r.ckpt, sizeof(float2) * 4 * nb * (n_seg + 1));
  if (e != cudaSuccess) return blobs_map_cuda(e);
  if (e == cudaSuccess) e = cudaMemsetAsync(r.ckpt, 0, sizeof(float2) * 4 * nb * (n_seg + 1), w->st());
  r.delta = delta;
  r.n_steps = n_steps;
  r.every = checkpoint_every;
  r.n_seg = n_seg;
  r.old_dt0 = w->old_dt;
  r.pending0 = w->pending;
  r.substeps = w->cfg.substeps;
  for (uint32_t g = 0; g <= n_seg; ++g) {
    float2* base = r.ckpt + 4 * nb * g;
    gather_state(w, base, base + nb, base + 2 * nb, base + 3 * nb);
    if (g == n_seg) break;
    const uint32_t steps = std::min(checkpoint_every, n_steps - g * checkpoint_every);
    int st = run_steps(w, delta, steps);
    if (st) return st;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return blobs_map_cuda(e);
  r.valid = true;
  return read_status(w);
}

int blobs_world_backward(blobs_world* w, const float* dl_dpos, float* dl_dvreq, float* dl_dk) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!w->loaded || !w->rec.valid || w->rec.substeps != w->cfg.substeps) return BLOBS_ERR_STATE;
  if (!dl_dpos) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaSetDevice(w->cfg.device);
  auto& r = w->rec;
  const size_t nb = w->nb;
  const uint32_t S = r.every * w->cfg.substeps;  // substeps per full segment
  cudaStream_t st = w->st();
  // scratch of the reverse pass: sized by a first carve, then carved
  const size_t slice = nb * sizeof(float2);
  struct Scratch {
    float2 *sp, *ss, *sv, *adj[2][4], *lpc, *la, *lv0;
    uint32_t* rec_list;
    uint32_t* rec_n;
    uint32_t* rec_max;
    float4* spr_terms;
    float* lk;
    Counters* saved;
  } x;
  auto lay = [&](Carver& cv) {
    x.sp = cv.take<float2>(nb * (S + 1));  // p, s, v of every recorded state
    x.ss = cv.take<float2>(nb * (S + 1));
    x.sv = cv.take<float2>(nb * (S + 1));
    x.rec_list = cv.take<uint32_t>((size_t)REC_CAP * nb * S);  // contacts of every body and substep
    x.rec_n = cv.take<uint32_t>(nb * S);
    x.rec_max = cv.take<uint32_t>(S);
    x.spr_terms = cv.take<float4>(w->ns ? w->ns : 1);
    for (int k = 0; k < 2; ++k)
      for (int m = 0; m < 4; ++m) x.adj[k][m] = cv.take<float2>(nb);  // adjoints of (p, po, s, v) in / out
    x.lpc = cv.take<float2>(nb);
    x.la = cv.take<float2>(nb);
    x.lv0 = cv.take<float2>(nb);
    x.lk = cv.take<float>(w->ns ? w->ns : 1);
    x.saved = cv.take<Counters>(1);
  };
  Carver sizer;
  lay(sizer);
  const size_t bytes = sizer.off;
  char* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes + 256);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  Carver cv;
  cv.base = buf;
  lay(cv);
  float2* const sp = x.sp;
  float2* const ss = x.ss;
  float2* const sv = x.sv;
  uint32_t* const rec_list = x.rec_list;
  uint32_t* const rec_n = x.rec_n;
  uint32_t* const rec_max = x.rec_max;
  float2* const lpc = x.lpc;
  float2* const la = x.la;
  float2* const lv0 = x.lv0;
  float* const lk = x.lk;
  Counters* const saved = x.saved;
  auto& adj = x.adj;
  e = cudaMemsetAsync(buf, 0, bytes, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(saved, w->dcounters, sizeof(Counters), cudaMemcpyDeviceToDevice, st);
  int in = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(adj[in][0], dl_dpos, slice, cudaMemcpyHostToDevice, st);
  const float dt_sub = (float)r.delta / (float)w->cfg.substeps;
  const uint32_t saved_timing = w->timing;
  w->timing = 0;
  // the recomputed substeps are not new collisions: no events
  w->dev.ev_rec = nullptr;
  int status = BLOBS_OK;
  std::vector<uint32_t> hmax(S);
  for (int g = (int)r.n_seg - 1; g >= 0 && e == cudaSuccess && status == BLOBS_OK; --g) {
    const uint32_t steps = std::min(r.every, r.n_steps - (uint32_t)g * r.every);
    const uint32_t nsub = steps * w->cfg.substeps;
    // restore the checkpoint and recompute the segment, recording every substep
    const float2* ck = r.ckpt + 4 * nb * g;
    restore_state(w, ck, ck + nb, ck + 2 * nb, ck + 3 * nb);
    w->old_dt = g == 0 ? r.old_dt0 : dt_sub;
    w->pending = g == 0 ? r.pending0 : false;
    cudaMemcpyAsync(sp, ck, slice, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(ss, ck + 2 * nb, slice, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(sv, ck + 3 * nb, slice, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(rec_max, 0, sizeof(uint32_t) * S, st);
    for (uint32_t t = 0; t < nsub; ++t) {
      w->rec_list = rec_list + (size_t)REC_CAP * nb * t;
      w->rec_n = rec_n + nb * t;
      w->rec_max = rec_max + t;
      const uint32_t sub = t % w->cfg.substeps;
      enqueue_substep(w, dt_sub, w->old_dt, w->pending, sub == 0, sub + 1 == w->cfg.substeps);
      w->pending = false;
      if (w->any_dynamic) w->old_dt = dt_sub;
      gather_state(w, sp + nb * (t + 1), nullptr, ss + nb * (t + 1), sv + nb * (t + 1));
    }
    w->rec_list = nullptr;
    w->rec_n = nullptr;
    w->rec_max = nullptr;
    e = cudaMemcpyAsync(hmax.data(), rec_max, sizeof(uint32_t) * nsub, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (uint32_t t = 0; t < nsub && e == cudaSuccess; ++t)
      if (hmax[t] > REC_CAP) status = BLOBS_ERR_OVERFLOW;  // a body with more contacts than recorded
    // reverse substeps of the segment
    for (int t = (int)nsub - 1; t >= 0 && status == BLOBS_OK; --t) {
      AdjointSubstep a;
      std::memset(&a, 0, sizeof(a));
      a.p_t = sp + nb * t;
      a.s_t = ss + nb * t;
      a.v_t = w->has_springs ? sv + nb * t : nullptr;
      a.p_t1 = sp + nb * (t + 1);
      a.s_t1 = ss + nb * (t + 1);
      a.rec_list = rec_list + (size_t)REC_CAP * nb * t;
      a.rec_n = rec_n + nb * t;
      a.spr_terms = x.spr_terms;
      a.lp_in = adj[in][0];
      a.lpo_in = adj[in][1];
      a.ls_in = adj[in][2];
      a.lv_in = adj[in][3];
      a.lp_out = adj[in ^ 1][0];
      a.lpo_out = adj[in ^ 1][1];
      a.ls_out = adj[in ^ 1][2];
      a.lv_out = adj[in ^ 1][3];
      a.lpc = lpc;
      a.la = la;
      a.lv0 = lv0;
      a.lk = lk;
      a.dt = dt_sub;
      a.ratio_first = dt_sub / r.old_dt0;
      a.first_substep = (g == 0 && t == 0) ? 1u : 0u;
      a.vreq_pending = (a.first_substep && r.pending0) ? 1u : 0u;
      launch_adjoint_substep(w->dev, a, st);
      in ^= 1;
    }
  }
  w->timing = saved_timing;
  w->attach_events();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess && status == BLOBS_OK) {
    if (dl_dvreq) e = cudaMemcpyAsync(dl_dvreq, lv0, slice, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && dl_dk && w->ns) e = cudaMemcpyAsync(dl_dk, lk, sizeof(float) * w->ns, cudaMemcpyDeviceToHost, st);
  }
  // errors flagged by the recomputed substeps stay sticky; then leave the
  // world in the rollout's final state, counters as after the forward pass
  if (e == cudaSuccess) {
    const int rs = read_status(w);
    if (rs && !status) status = rs;
    const float2* fin = r.ckpt + 4 * nb * r.n_seg;
    restore_state(w, fin, fin + nb, fin + 2 * nb, fin + 3 * nb);
    w->old_dt = dt_sub;
    w->pending = false;
    e = cudaMemcpyAsync(w->dcounters, saved, sizeof(Counters), cudaMemcpyDeviceToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  if (status) return status;
  return read_status(w);
}

int blobs_world_set_events(blobs_world* w, int enabled, uint32_t capacity) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (enabled && (capacity == 0 || capacity > 0x7fffffffu)) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  cudaStream_t st = w->st();
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  const bool was_on = w->events_on;
  w->drop_graphs();  // the event pointers and the fusion choice are baked into graphs
  w->drop_recording();  // checkpoints hold V in the previous mode
  if (w->ev_mem) cudaFree(w->ev_mem);
  w->ev_mem = nullptr;
  w->ev_host.clear();
  w->events_on = false;
  if (enabled) {
    Carver sizer;
    auto lay = [&](Carver& cv) {
      w->ev_rec = cv.take<uint4>(capacity);
      w->ev_vel = cv.take<float4>(capacity);
      w->ev_count = cv.take<uint32_t>(2);  // count, then the substep sequence
    };
    lay(sizer);
    e = cudaMalloc(&w->ev_mem, sizer.off + 256);
    if (e != cudaSuccess) {
      w->ev_mem = nullptr;
      w->attach_events();
      return blobs_map_cuda(e);
    }
    Carver cv;
    cv.base = static_cast<char*>(w->ev_mem);
    lay(cv);
    w->ev_seq = w->ev_count + 1;
    w->ev_cap = capacity;
    e = cudaMemsetAsync(w->ev_count, 0, 2 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return blobs_map_cuda(e);
    w->events_on = true;
  }
  if (w->loaded && w->sorted_storage && !w->has_springs && w->events_on != was_on) {
    const int c = (int)w->cur;
    if (w->events_on) {
      // V becomes calculated_velocity, double-buffered with the state
      if (w->vbuf != c) e = cudaMemcpyAsync(w->dev.sv[c], w->dev.sv[w->vbuf], sizeof(float2) * w->nb,
                                            cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess && w->v_div != 0.0f) launch_v_divide(w->dev.sv[c], w->nb, w->v_div, st);
    }
    w->vbuf = c;
    w->v_div = 0.0f;
  }
  w->attach_events();
  if (e == cudaSuccess) e = cudaGetLastError();
  return blobs_map_cuda(e);
}

int blobs_world_drain_events(blobs_world* w, uint32_t* col_a, uint32_t* col_b, float* impact_vel_a,
                             float* impact_vel_b, uint64_t cap, uint64_t* n_written, uint64_t* n_left) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!n_written || (cap && (!col_a || !col_b))) return BLOBS_ERR_INVALID_ARGUMENT;
  *n_written = 0;
  if (n_left) *n_left = 0;
  if (!w->events_on) return BLOBS_ERR_STATE;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  cudaStream_t st = w->st();
  uint32_t head[2] = {0, 0};
  e = cudaMemcpyAsync(head, w->ev_count, sizeof(head), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  const uint32_t n = head[0];
  if (n > w->ev_cap) {
    // the appended subset is not a prefix of the reference order: drop it
    e = cudaMemsetAsync(w->ev_count, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (n_left) *n_left = n;
    return e == cudaSuccess ? BLOBS_ERR_OVERFLOW : blobs_map_cuda(e);
  }
  if (n) {
    std::vector<uint4> rec(n);
    std::vector<float4> vel(n);
    e = cudaMemcpyAsync(rec.data(), w->ev_rec, sizeof(uint4) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vel.data(), w->ev_vel, sizeof(float4) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w->ev_count, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return blobs_map_cuda(e);
    // the reference's order: substep by substep, outer collider ascending,
    // inner collider ascending (physics.rs:247-248)
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
      const uint4 &p = rec[x], &q = rec[y];
      if (p.x != q.x) return (int32_t)(p.x - q.x) < 0;  // sequence, modulo 2^32
      if (p.y != q.y) return p.y < q.y;
      return p.z < q.z;
    });
    for (uint32_t k : order) {
      blobs_world::HostEvent ev;
      ev.a = rec[k].y;
      ev.b = rec[k].z;
      ev.va[0] = vel[k].x;
      ev.va[1] = vel[k].y;
      ev.vb[0] = vel[k].z;
      ev.vb[1] = vel[k].w;
      w->ev_host.push_back(ev);
    }
  }
  uint64_t k = 0;
  while (k < cap && !w->ev_host.empty()) {
    const blobs_world::HostEvent& ev = w->ev_host.front();
    col_a[k] = ev.a;
    col_b[k] = ev.b;
    if (impact_vel_a) impact_vel_a[2 * k] = ev.va[0], impact_vel_a[2 * k + 1] = ev.va[1];
    if (impact_vel_b) impact_vel_b[2 * k] = ev.vb[0], impact_vel_b[2 * k + 1] = ev.vb[1];
    w->ev_host.pop_front();
    ++k;
  }
  *n_written = k;
  if (n_left) *n_left = w->ev_host.size();
  return read_status(w);
}

int blobs_world_autotune(blobs_world* w, const blobs_scene* scene, float old_dt, double delta, uint32_t trial_steps,
                         float* cell_scale) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!scene || trial_steps == 0 || !(delta > 0.0)) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(w->cfg.device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  // every cell edge >= the smallest exact one gives the same contacts in the
  // same order, so the choice only changes the time
  static const float kScales[] = {1.0f, 1.125f, 1.25f, 1.5f, 1.75f};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms = INFINITY, best = 1.0f;
  int status = BLOBS_OK;
  for (float sc : kScales) {
    w->cell_scale = sc;
    status = blobs_world_load(w, scene, old_dt);
    if (status) break;
    status = run_steps(w, delta, 2);  // the irregular first step, graph capture
    if (!status) status = run_steps(w, delta, trial_steps);  // captures the trial graph
    if (status) break;
    e = cudaEventRecord(e0, w->st());
    if (e == cudaSuccess) status = run_steps(w, delta, trial_steps);
    if (e == cudaSuccess && !status) e = cudaEventRecord(e1, w->st());
    if (e == cudaSuccess && !status) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess && !status) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) status = blobs_map_cuda(e);
    if (!status) status = read_status(w);
    if (status) break;
    if (ms < best_ms) {
      best_ms = ms;
      best = sc;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  w->cell_scale = best;
  if (status) return status;
  if (cell_scale) *cell_scale = best;
  return blobs_world_load(w, scene, old_dt);  // the scene's initial state, tuned grid
}

int blobs_world_kernel_launches(blobs_world* w, uint64_t* count) {
  if (!w || !count) return BLOBS_ERR_INVALID_HANDLE;
  *count = w->kernels_launched;
  return BLOBS_OK;
}

int blobs_world_set_timing(blobs_world* w, int enabled) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (enabled < 0 || enabled > 2) return BLOBS_ERR_INVALID_ARGUMENT;
  w->timing = (uint32_t)enabled;
  return BLOBS_OK;
}

int blobs_world_phase_times(blobs_world* w, double* ms, uint64_t* launches, uint32_t n_phases) {
  if (!w) return BLOBS_ERR_INVALID_HANDLE;
  if (!ms || !launches || n_phases < N_PHASES) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaSetDevice(w->cfg.device);
  cudaError_t e = cudaStreamSynchronize(w->st());
  if (e != cudaSuccess) return blobs_map_cuda(e);
  for (uint32_t p = 0; p < n_phases; ++p) ms[p] = 0.0, launches[p] = 0;
  for (TimingSet* ts : w->launched_sets)
    for (auto& m : ts->marks) {
      float t = 0.0f;
      if (cudaEventElapsedTime(&t, m.a, m.b) == cudaSuccess) {
        ms[m.phase] += t;
        launches[m.phase] += 1;
      }
    }
  w->launched_sets.clear();
  w->eager_timing.destroy();
  return BLOBS_OK;
}

int blobs_body_mass_inertia(uint32_t n_bodies, uint32_t n_colliders, const uint32_t* col_parent,
                            const float* col_offset, const float* col_radius, const float* col_mass_override,
                            const uint8_t* col_sensor, float* mass_out, float* inertia_out) {
  if (!mass_out || !inertia_out) return BLOBS_ERR_INVALID_ARGUMENT;
  if (n_colliders && (!col_parent || !col_radius)) return BLOBS_ERR_INVALID_ARGUMENT;
  std::vector<float> m(n_bodies, 0.0f), I(n_bodies, 0.0f);
  std::vector<uint8_t> has(n_bodies, 0);
  for (uint32_t c = 0; c < n_colliders; ++c)
    if (col_parent[c] >= n_bodies) return BLOBS_ERR_INVALID_ARGUMENT;
  // Each handle sits twice in the body's collider list (collider.rs:180 and
  // physics.rs:144); the sum runs over that list in order.
  for (uint32_t c = 0; c < n_colliders; ++c) {
    const uint32_t b = col_parent[c];
    has[b] = 1;
    if (col_sensor && col_sensor[c]) continue;
    const float r = col_radius[c];
    const float cm = (col_mass_override && !std::isnan(col_mass_override[c])) ? col_mass_override[c] : r * 2.0f;
    const float2 off = col_offset ? v2(col_offset[2 * c], col_offset[2 * c + 1]) : v2(0.0f, 0.0f);
    const float d = len2(off);
    float ci = 0.5f * cm * (r * r);
    ci = ci + cm * (d * d);
    for (int twice = 0; twice < 2; ++twice) {
      m[b] = m[b] + cm;
      I[b] = I[b] + ci;
    }
  }
  for (uint32_t b = 0; b < n_bodies; ++b) {
    if (!has[b]) {
      mass_out[b] = 1.0f;  // RigidBodyBuilder::build default (rigid_body.rs:385,388)
      inertia_out[b] = 1.0f;
      continue;
    }
    mass_out[b] = m[b] == 0.0f ? 1.0f : m[b];
    inertia_out[b] = I[b] == 0.0f ? 1.0f : I[b];
  }
  return BLOBS_OK;
}

}  // extern "C"
