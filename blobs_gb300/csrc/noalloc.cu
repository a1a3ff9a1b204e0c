// noalloc.cu -- contact-pair emission that allocates no memory.
//
// blobs_contact_pairs_noalloc computes the same contact pair set as
// blobs_world_emit_pairs(contacts_only = 1) -- every collider pair with
// different parents, passing InteractionGroups::test and closer than the sum
// of the radii (the pair set of physics.rs:248-269) -- for colliders the
// caller already holds in device memory, without a world and without any
// allocation.  It is for callers that must not allocate device memory while
// they run: a host whose frame loop cannot absorb cudaMalloc / cudaFree
// (both synchronise the whole device), or a host whose device memory is
// owned and budgeted by its own allocator.  Every scratch buffer it needs
// lives in one file-scope device array, g_noalloc_scratch, sized for at most
// NA_MAX_COLLIDERS colliders and NA_MAX_CELLS grid cells; every GPU that
// loads this library holds that array until the process exits.
#include <mutex>

#include "blobs_gpu.h"
#include "device.cuh"
#include "world.h"

namespace {

constexpr uint32_t NA_MAX_COLLIDERS = 1u << 16;  // 65,536 colliders
constexpr uint32_t NA_LOG2_MAX_CELLS = 17;       // 131,072 grid cells
constexpr uint32_t NA_MAX_CELLS = 1u << NA_LOG2_MAX_CELLS;
constexpr uint32_t NA_SCAN_THREADS = 1024;
constexpr uint32_t NA_MAX_DEVICES = 64;

// Layout of the scratch array (byte offsets, each 256-byte aligned).
constexpr size_t NA_OFF_HDR = 0;                                                // 8 x u32 header
constexpr size_t NA_OFF_COUNT = 256;                                            // u32[NA_MAX_CELLS]
constexpr size_t NA_OFF_START = NA_OFF_COUNT + 4ull * NA_MAX_CELLS;             // u32[NA_MAX_CELLS + 1]
constexpr size_t NA_OFF_RANK = NA_OFF_START + 4ull * NA_MAX_CELLS + 256;        // u32[NA_MAX_COLLIDERS]
constexpr size_t NA_OFF_KEY = NA_OFF_RANK + 4ull * NA_MAX_COLLIDERS;            // u32[NA_MAX_COLLIDERS]
constexpr size_t NA_OFF_SORTED = NA_OFF_KEY + 4ull * NA_MAX_COLLIDERS;          // float4[NA_MAX_COLLIDERS]
constexpr size_t NA_SCRATCH_BYTES = NA_OFF_SORTED + 16ull * NA_MAX_COLLIDERS;   // ~2.3 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

struct Scratch {
  uint32_t* hdr;  // [0..3] ordered bounds (min x, min y, max x, max y), [4] max radius bits
  uint32_t* count;
  uint32_t* start;
  uint32_t* rank;
  uint32_t* key;
  float4* sorted;
};

__host__ __device__ inline Scratch carve(unsigned char* base) {
  Scratch s;
  s.hdr = reinterpret_cast<uint32_t*>(base + NA_OFF_HDR);
  s.count = reinterpret_cast<uint32_t*>(base + NA_OFF_COUNT);
  s.start = reinterpret_cast<uint32_t*>(base + NA_OFF_START);
  s.rank = reinterpret_cast<uint32_t*>(base + NA_OFF_RANK);
  s.key = reinterpret_cast<uint32_t*>(base + NA_OFF_KEY);
  s.sorted = reinterpret_cast<float4*>(base + NA_OFF_SORTED);
  return s;
}

// Monotone map of floats to unsigned ints (for atomicMin / atomicMax).
__device__ inline uint32_t ordered(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ inline float unordered(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

struct Grid {
  float cs, inv, ox, oy;
  uint32_t log2w, log2h;
};

// The grid every kernel derives from the header: cell = 2 rmax (1 + 1/64),
// origin one cell before the extent, power-of-two sides capped to
// NA_MAX_CELLS cells (coordinates wrap beyond, which keeps the 3x3 search
// exact; blobs::grid_coord keeps it exact at any distance from the origin).
__device__ inline Grid grid_of(const uint32_t* hdr) {
  Grid g;
  const float rmax = __uint_as_float(hdr[4]);
  g.cs = rmax > 0.0f ? 2.0f * rmax * (1.0f + 1.0f / 64.0f) : 1.0f;
  g.inv = 1.0f / g.cs;
  const float lo_x = unordered(hdr[0]), lo_y = unordered(hdr[1]);
  const float hi_x = unordered(hdr[2]), hi_y = unordered(hdr[3]);
  const bool finite = lo_x <= hi_x && lo_y <= hi_y;
  g.ox = finite ? lo_x - g.cs : 0.0f;
  g.oy = finite ? lo_y - g.cs : 0.0f;
  uint32_t lw = 2, lh = 2;
  if (finite) {
    const float ex = (hi_x - lo_x) * g.inv + 3.0f, ey = (hi_y - lo_y) * g.inv + 3.0f;
    while (lw < 30 && (float)(1u << lw) < ex) ++lw;
    while (lh < 30 && (float)(1u << lh) < ey) ++lh;
  }
  while (lw + lh > NA_LOG2_MAX_CELLS) {
    if (lw >= lh && lw > 2) --lw;
    else if (lh > 2) --lh;
    else break;
  }
  g.log2w = lw;
  g.log2h = lh;
  return g;
}

__device__ inline uint32_t key_of(const Grid& g, float x, float y) {
  const uint32_t ix = (uint32_t)blobs::grid_coord(x, g.ox, g.inv) & ((1u << g.log2w) - 1u);
  const uint32_t iy = (uint32_t)blobs::grid_coord(y, g.oy, g.inv) & ((1u << g.log2h) - 1u);
  return (iy << g.log2w) | ix;
}

__global__ void na_init(Scratch s, unsigned long long* count) {
  if (threadIdx.x == 0) {
    s.hdr[0] = s.hdr[1] = 0xffffffffu;  // min bounds
    s.hdr[2] = s.hdr[3] = 0u;           // max bounds
    s.hdr[4] = 0u;                      // max radius (bits of a non-negative float)
    *count = 0ull;
  }
}

__global__ void na_bounds(Scratch s, uint32_t n, const float2* __restrict__ snap, const float* __restrict__ radius) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 p = snap[i];
  if (isfinite(p.x) && isfinite(p.y)) {
    atomicMin(s.hdr + 0, ordered(p.x));
    atomicMin(s.hdr + 1, ordered(p.y));
    atomicMax(s.hdr + 2, ordered(p.x));
    atomicMax(s.hdr + 3, ordered(p.y));
  }
  // +inf counts (every collider then shares one cell, as in the world
  // path); NaN never passes the contact test and is left out
  const float r = radius[i];
  if (r > 0.0f) atomicMax(s.hdr + 4, __float_as_uint(r));
}

__global__ void na_keys(Scratch s, uint32_t n, const float2* __restrict__ snap) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Grid g = grid_of(s.hdr);
  const float2 p = snap[i];
  const uint32_t k = key_of(g, p.x, p.y);
  s.key[i] = k;
  s.rank[i] = atomicAdd(s.count + k, 1u);
}

// One block scans all cells (at most NA_MAX_CELLS): start[k] = sum(count[0..k)).
__global__ void __launch_bounds__(NA_SCAN_THREADS) na_scan(Scratch s) {
  __shared__ uint32_t s_warp[NA_SCAN_THREADS / 32];
  const Grid g = grid_of(s.hdr);
  const uint32_t cells = 1u << (g.log2w + g.log2h);
  const uint32_t per = (cells + NA_SCAN_THREADS - 1) / NA_SCAN_THREADS;
  const uint32_t k0 = threadIdx.x * per, k1 = min(k0 + per, cells);
  uint32_t sum = 0;
  for (uint32_t k = k0; k < k1; ++k) sum += s.count[k];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = s_warp[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (uint32_t)o) t += y;
    }
    s_warp[lane] = t;
  }
  __syncthreads();
  uint32_t run = (warp ? s_warp[warp - 1] : 0u) + x - sum;
  for (uint32_t k = k0; k < k1; ++k) {
    s.start[k] = run;
    run += s.count[k];
  }
  if (threadIdx.x == NA_SCAN_THREADS - 1) s.start[cells] = run;
}

__global__ void na_scatter(Scratch s, uint32_t n, const float2* __restrict__ snap, const float* __restrict__ radius) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t slot = s.start[s.key[i]] + s.rank[i];
  if (slot >= n) return;
  const float2 p = snap[i];
  s.sorted[slot] = make_float4(p.x, p.y, radius[i], __uint_as_float(i));
}

// Contact pairs (hi, lo), hi > lo, of the reference's filters and test.
__global__ void na_emit(Scratch s, uint32_t n, const uint32_t* __restrict__ parent, const uint32_t* __restrict__ memb,
                        const uint32_t* __restrict__ filt, uint32_t* __restrict__ pairs, unsigned long long cap,
                        unsigned long long* __restrict__ count) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const Grid g = grid_of(s.hdr);
  const float4 me = s.sorted[e];
  const uint32_t c = __float_as_uint(me.w);
  if (c >= n) return;
  const uint32_t wm = (1u << g.log2w) - 1u, hm = (1u << g.log2h) - 1u;
  const uint32_t ix = (uint32_t)blobs::grid_coord(me.x, g.ox, g.inv), iy = (uint32_t)blobs::grid_coord(me.y, g.oy, g.inv);
  for (int oy = -1; oy <= 1; ++oy) {
    const uint32_t row = ((iy + (uint32_t)oy) & hm) << g.log2w;
    for (int ox = -1; ox <= 1; ++ox) {
      const uint32_t cell = row | ((ix + (uint32_t)ox) & wm);
      const uint32_t q1 = min(s.start[cell + 1], n);
      for (uint32_t q = s.start[cell]; q < q1; ++q) {
        const float4 o = s.sorted[q];
        const uint32_t c2 = __float_as_uint(o.w);
        if (c2 >= c) continue;
        if (parent && parent[c] == parent[c2]) continue;
        const uint32_t m1 = memb ? memb[c] : 0xffffffffu, f1 = filt ? filt[c] : 0xffffffffu;
        const uint32_t m2 = memb ? memb[c2] : 0xffffffffu, f2 = filt ? filt[c2] : 0xffffffffu;
        if (!((m1 & f2) != 0u && (m2 & f1) != 0u)) continue;
        const float dx = me.x - o.x, dy = me.y - o.y;
        if (!(sqrtf((dx * dx) + (dy * dy)) < me.z + o.z)) continue;
        const unsigned long long k = atomicAdd(count, 1ull);
        if (k < cap) {
          pairs[2 * k] = c;
          pairs[2 * k + 1] = c2;
        }
      }
    }
  }
}

std::mutex g_setup_mutex;
void* g_scratch_ptr[NA_MAX_DEVICES] = {};

}  // namespace

extern "C" {

uint32_t blobs_noalloc_max_colliders(void) { return NA_MAX_COLLIDERS; }

int blobs_contact_pairs_noalloc(uint32_t n, const float* snap, const float* radius, const uint32_t* parent,
                                const uint32_t* memb, const uint32_t* filt, uint32_t* pairs, uint64_t cap,
                                unsigned long long* count, void* stream) {
  if (n > NA_MAX_COLLIDERS) return BLOBS_ERR_INVALID_ARGUMENT;  // beyond the static scratch
  if (!count || (n && (!snap || !radius)) || (cap && !pairs)) return BLOBS_ERR_INVALID_ARGUMENT;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  if (dev < 0 || dev >= (int)NA_MAX_DEVICES) return BLOBS_ERR_INVALID_ARGUMENT;
  void* base = nullptr;
  {
    // first call on a device: look up the device address of the scratch array
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      e = cudaGetSymbolAddress(&g_scratch_ptr[dev], g_noalloc_scratch);
      if (e != cudaSuccess) {
        g_scratch_ptr[dev] = nullptr;
        return blobs_map_cuda(e);
      }
    }
    base = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Scratch s = carve(static_cast<unsigned char*>(base));
  // the counts must start at zero; the rest is overwritten before it is read
  e = cudaMemsetAsync(s.count, 0, 4ull * NA_MAX_CELLS, st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  na_init<<<1, 32, 0, st>>>(s, count);
  if (n) {
    const uint32_t blocks = (n + 255u) / 256u;
    const float2* p = reinterpret_cast<const float2*>(snap);
    na_bounds<<<blocks, 256, 0, st>>>(s, n, p, radius);
    na_keys<<<blocks, 256, 0, st>>>(s, n, p);
    na_scan<<<1, NA_SCAN_THREADS, 0, st>>>(s);
    na_scatter<<<blocks, 256, 0, st>>>(s, n, p, radius);
    na_emit<<<blocks, 256, 0, st>>>(s, n, parent, memb, filt, pairs, cap, count);
  }
  return blobs_map_cuda(cudaGetLastError());
}

}  // extern "C"
