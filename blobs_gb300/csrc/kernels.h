// kernels.h -- host-side launchers of the substep kernels (kernels.cu).
#pragma once

#include "device.cuh"

namespace blobs {

void launch_keys(const WorldDev& w, bool multiworld, cudaStream_t st);
void launch_scan(const WorldDev& w, cudaStream_t st);
void launch_scatter_forces(const WorldDev& w, const float2* pos, bool multiworld, bool scatter, bool springs,
                           bool pending, cudaStream_t st);
void launch_contacts(const WorldDev& w, const float2* pos_in, float2* pos_out, bool multiworld, bool single,
                     bool springs, bool pending, bool fuse, float dt, float old_dt, bool do_keys, bool rot_dynamic,
                     cudaStream_t st);
void launch_joints(const WorldDev& w, float2* pos, uint32_t j0, uint32_t j1, float dt, cudaStream_t st);
void launch_integrate(const WorldDev& w, const float2* pos_in, float2* pos_out, bool multiworld, bool single,
                      bool springs, bool pending, float dt, float old_dt, bool do_keys, bool rot_dynamic,
                      cudaStream_t st);

}  // namespace blobs
