// world.h -- internal accessors shared between the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

struct blobs_world;

int blobs_map_cuda(cudaError_t e);
const blobs::WorldDev* blobs_world_dev(blobs_world* w);
cudaStream_t blobs_world_stream(blobs_world* w);
float2* blobs_world_pos(blobs_world* w);
