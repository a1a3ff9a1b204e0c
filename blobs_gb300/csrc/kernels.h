// kernels.h -- host-side launchers of the substep kernels (kernels.cu).
#pragma once

#include "device.cuh"

namespace blobs {

void launch_keys(const WorldDev& w, bool multiworld, cudaStream_t st);
// the cell scan; returns the number of kernels it launched
uint32_t launch_scan(const WorldDev& w, cudaStream_t st);
void launch_scatter_forces(const WorldDev& w, const float2* pos, bool multiworld, bool scatter, bool springs,
                           bool pending, cudaStream_t st);
uint32_t launch_contacts(const WorldDev& w, const float2* pos_in, float2* pos_out, bool multiworld, bool single,
                     bool springs, bool pending, bool fuse, float dt, float old_dt, bool do_keys, bool rot_dynamic,
                     cudaStream_t st);
void launch_joints(const WorldDev& w, float2* pos, uint32_t j0, uint32_t j1, float dt, cudaStream_t st);
void launch_joint_blocks(const WorldDev& w, float2* pos, float dt, uint32_t iterations, cudaStream_t st);
void launch_ev_tick(const WorldDev& w, cudaStream_t st);
void launch_v_divide(float2* v, uint32_t n, float dt, cudaStream_t st);
void launch_integrate(const WorldDev& w, const float2* pos_in, float2* pos_out, bool multiworld, bool single,
                      bool springs, bool pending, float dt, float old_dt, bool do_keys, bool rot_dynamic,
                      cudaStream_t st);

void launch_emit_pairs(const WorldDev& w, bool multiworld, uint32_t mode, uint32_t* out, unsigned long long cap,
                       unsigned long long* count, cudaStream_t st);

// single-sphere path with cell-sorted storage (single.cu); mode 0: one
// uniform world, 1: one world with per-body records, 2: batched worlds
void launch_permute(const WorldDev& w, const SingleArgs& a, cudaStream_t st);
void launch_scatter_cand(const WorldDev& w, const float4* a_in, float4* cand, cudaStream_t st);
void launch_step_single(const WorldDev& w, const SingleArgs& a, int mode, cudaStream_t st);
// the bodies the plain step deferred (after launch_step_single, same args)
void launch_step_deferred(const WorldDev& w, const SingleArgs& a, int mode, cudaStream_t st);
void launch_keys_single(const WorldDev& w, const float4* A, int mode, cudaStream_t st);
void launch_gather_single(const WorldDev& w, const float4* A, const float4* B, const float2* V, float2* pos,
                          float2* pos_old, float2* vel, float2* snap, float v_div, cudaStream_t st);
void launch_write_single(const WorldDev& w, float4* A, float4* B, float2* V, const float2* pos,
                         const float2* pos_old, const float2* vel, const float2* snap, cudaStream_t st);

// adjoint of the single-sphere substep (adjoint.cu)
struct AdjointSubstep {
  // recorded state at the start of the substep (t) and after it (t + 1), arena order
  const float2* p_t;
  const float2* s_t;
  const float2* v_t;
  const float2* p_t1;
  const float2* s_t1;
  const uint32_t* rec_list;  // contacts of each body in the substep, as recorded (REC_CAP x n_bodies)
  const uint32_t* rec_n;     // per body: recorded contacts
  // adjoints of the state after the substep (in) and before it (out)
  const float2* lp_in;
  const float2* lpo_in;
  const float2* ls_in;
  const float2* lv_in;
  float2* lp_out;
  float2* lpo_out;
  float2* ls_out;
  float2* lv_out;
  float2* lpc;             // scratch: adjoint of the post-contact position
  float2* la;              // scratch: adjoint of the acceleration
  float2* lv0;             // gradient of the velocity requests (first substep of the rollout)
  float* lk;               // gradient of the spring stiffnesses (accumulated)
  float4* spr_terms;       // scratch: per spring, the adjoint of d (pb - pa) and of rv (va - vb)
  float dt;
  float ratio_first;       // dt / old_dt for the first dynamic body (first substep only)
  uint32_t first_substep;  // the rollout's first substep (dt / old_dt applies)
  uint32_t vreq_pending;   // velocity requests were pending at the rollout's start
};
void launch_adjoint_substep(const WorldDev& w, const AdjointSubstep& a, cudaStream_t st);

}  // namespace blobs
