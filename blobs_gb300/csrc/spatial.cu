// spatial.cu -- SpatialHash (blobs/src/spatial.rs) on the device: a point set
// with ids and radii, bucketed by integer cell, and SpatialHash::query as a
// batched radius query.
//
// The reference keys an unbounded HashMap by the cell (i32, i32) =
// ((x / cs).floor() as i32, (y / cs).floor() as i32) (spatial.rs:57-62) and a
// query visits the 3x3 cells around the query point's cell, keeping every
// point with |p - q|^2 <= (query_radius + radius)^2 (spatial.rs:155-195) --
// points further than one cell away are never seen, whatever the radius.
// Here the cells are hashed into a power-of-two table of buckets (>= 2 per
// point), points are counting-sorted by bucket, and a query walks the nine
// buckets of its neighbour cells, keeping only points whose own cell is that
// neighbour cell: buckets shared by several cells cost time, never results.
// Results of one query are returned in ascending id (the reference's order is
// its HashMap's iteration order, which is unspecified).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "blobs_gpu.h"
#include "device.cuh"
#include "kernels.h"
#include "world.h"

using namespace blobs;

namespace {

__device__ __forceinline__ uint32_t cell_hash(int32_t cx, int32_t cy) {
  // two odd multipliers and a final avalanche (a 32-bit integer mix)
  uint32_t h = (uint32_t)cx * 0x9E3779B1u ^ ((uint32_t)cy * 0x85EBCA77u + 0x165667B1u);
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return h;
}

struct HashDev {
  uint32_t n, mask;  // points, buckets - 1
  float cs;
  const float2* xy;
  const float* radius;
  int2* cell;
  uint32_t* bucket;
  uint32_t* rank;
  uint32_t* count;   // per bucket, zero between builds
  uint32_t* start;   // per bucket + 1
  uint32_t* sorted;  // point indices, bucket order
};

__global__ void __launch_bounds__(256) k_sh_keys(HashDev h) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= h.n) return;
  const float2 p = h.xy[i];
  const int2 c = make_int2(cell_coord(p.x, h.cs), cell_coord(p.y, h.cs));
  h.cell[i] = c;
  const uint32_t b = cell_hash(c.x, c.y) & h.mask;
  h.bucket[i] = b;
  h.rank[i] = atomicAdd(h.count + b, 1u);
}

__global__ void __launch_bounds__(256) k_sh_scatter(HashDev h, uint32_t* status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= h.n) return;
  const uint32_t s = h.start[h.bucket[i]] + h.rank[i];
  if (s >= h.n) {
    atomicOr(status, ST_BAD_INDEX);
    return;
  }
  h.sorted[s] = i;
}

// In-place heap sort of a[0..n) (ascending).
__device__ void heap_sort(unsigned long long* a, uint32_t n) {
  auto sift = [&](uint32_t root, uint32_t end) {
    while (true) {
      uint32_t child = 2u * root + 1u;
      if (child >= end) return;
      if (child + 1u < end && a[child] < a[child + 1u]) ++child;
      if (!(a[root] < a[child])) return;
      const unsigned long long t = a[root];
      a[root] = a[child];
      a[child] = t;
      root = child;
    }
  };
  if (n < 2u) return;
  for (uint32_t k = n / 2u; k-- > 0u;) sift(k, n);
  for (uint32_t end = n - 1u; end > 0u; --end) {
    const unsigned long long t = a[0];
    a[0] = a[end];
    a[end] = t;
    sift(0u, end);
  }
}

// One thread per query.  WRITE = false: count the matches into qcount;
// WRITE = true: write their ids from qstart[q] on and sort them.
template <bool WRITE>
__global__ void __launch_bounds__(256) k_sh_query(HashDev h, const unsigned long long* __restrict__ ids,
                                                  uint32_t nq, const float2* __restrict__ qxy,
                                                  const float* __restrict__ qr, uint32_t* qcount,
                                                  const uint32_t* qstart, unsigned long long* out,
                                                  unsigned long long cap) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const float2 x = qxy[q];
  const float r = qr[q];
  const int32_t cx = cell_coord(x.x, h.cs), cy = cell_coord(x.y, h.cs);
  uint32_t k = 0;
  const unsigned long long base = WRITE ? qstart[q] : 0ull;
  // spatial.rs:139-153: the 3x3 neighbour cells (i32 arithmetic, wrapping)
  for (int dx = -1; dx <= 1; ++dx) {
    for (int dy = -1; dy <= 1; ++dy) {
      const int32_t nx = (int32_t)((uint32_t)cx + (uint32_t)dx), ny = (int32_t)((uint32_t)cy + (uint32_t)dy);
      const uint32_t b = cell_hash(nx, ny) & h.mask;
      const uint32_t s1 = h.start[b + 1u];
      for (uint32_t s = h.start[b]; s < s1; ++s) {
        const uint32_t i = h.sorted[s];
        const int2 c = h.cell[i];
        if (c.x != nx || c.y != ny) continue;
        const float2 p = h.xy[i];
        const float dist = r + h.radius[i];
        const float ex = p.x - x.x, ey = p.y - x.y;
        if ((ex * ex) + (ey * ey) <= dist * dist) {
          if (WRITE && base + k < cap) out[base + k] = ids[i];
          ++k;
        }
      }
    }
  }
  if (!WRITE) {
    qcount[q] = k;
  } else if (base + k <= cap) {
    heap_sort(out + base, k);
  }
}

inline uint32_t nblk(uint64_t n) { return (uint32_t)((n + 255u) / 256u); }

// The two-kernel cell scan of kernels.cu over an arbitrary count array:
// start[k] = sum(count[0..k)), start[n] = total, count zeroed.
void scan_counts(uint32_t* count, uint32_t* start, uint32_t n, uint32_t* tile_sums, uint32_t* sub_bins,
                 cudaStream_t st) {
  WorldDev d{};
  d.cell_count = count;
  d.cell_start = start;
  d.n_cells = n;
  d.n_tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  d.tile_sums = tile_sums;
  d.contacts_sub = sub_bins;
  d.defer_sub = sub_bins;
  launch_scan(d, st);
}

}  // namespace

struct blobs_spatial_hash {
  float cs = 1.0f;
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t n = 0, n_buckets = 0;
  // points: ids, xy, radius, cell, bucket, rank, sorted; buckets: count, start;
  // scan scratch
  void* pts = nullptr;
  size_t pts_bytes = 0;
  unsigned long long* ids = nullptr;
  float2* xy = nullptr;
  float* radius = nullptr;
  int2* cell = nullptr;
  uint32_t *bucket = nullptr, *rank = nullptr, *sorted = nullptr, *count = nullptr, *start = nullptr;
  uint32_t *tile_sums = nullptr, *sub_bins = nullptr, *status = nullptr;
  // queries
  void* qmem = nullptr;
  size_t qmem_bytes = 0;
  void* omem = nullptr;
  size_t omem_bytes = 0;

  HashDev dev() const {
    HashDev h;
    h.n = n;
    h.mask = n_buckets ? n_buckets - 1u : 0u;
    h.cs = cs;
    h.xy = xy;
    h.radius = radius;
    h.cell = cell;
    h.bucket = bucket;
    h.rank = rank;
    h.count = count;
    h.start = start;
    h.sorted = sorted;
    return h;
  }
  ~blobs_spatial_hash() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    if (pts) cudaFree(pts);
    if (qmem) cudaFree(qmem);
    if (omem) cudaFree(omem);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

struct Carve {
  size_t off = 0;
  char* base = nullptr;
  template <class T> T* take(size_t count) {
    const size_t at = (off + 255) & ~(size_t)255;
    off = at + (count ? count * sizeof(T) : 1);
    return base ? reinterpret_cast<T*>(base + at) : nullptr;
  }
};

// (Re)allocates `mem` to hold `bytes` when it is smaller.
cudaError_t ensure(void** mem, size_t* have, size_t bytes) {
  if (*have >= bytes && *mem) return cudaSuccess;
  if (*mem) cudaFree(*mem);
  *mem = nullptr;
  *have = 0;
  cudaError_t e = cudaMalloc(mem, bytes);
  if (e == cudaSuccess) *have = bytes;
  return e;
}

}  // namespace

extern "C" {

int blobs_spatial_hash_create(float cell_size, int32_t device, blobs_spatial_hash** out) {
  if (!out) return BLOBS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!(cell_size > 0.0f) || !std::isfinite(cell_size)) return BLOBS_ERR_INVALID_ARGUMENT;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) {
    cudaGetLastError();
    return BLOBS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= nd) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  blobs_spatial_hash* h = new blobs_spatial_hash();
  h->cs = cell_size;
  h->device = device;
  e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return blobs_map_cuda(e);
  }
  *out = h;
  return BLOBS_OK;
}

int blobs_spatial_hash_destroy(blobs_spatial_hash* h) {
  if (!h) return BLOBS_ERR_INVALID_HANDLE;
  delete h;
  return BLOBS_OK;
}

int blobs_spatial_hash_set_points(blobs_spatial_hash* h, uint64_t n, const uint64_t* ids, const float* xy,
                                  const float* radius) {
  if (!h) return BLOBS_ERR_INVALID_HANDLE;
  if (n && (!ids || !xy || !radius)) return BLOBS_ERR_INVALID_ARGUMENT;
  if (n > 0x3fffffffull) return BLOBS_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  cudaStream_t st = h->stream;
  uint32_t nb = 1024;
  while (nb < 2 * n) nb <<= 1;
  const uint32_t n_tiles = (nb + SCAN_TILE - 1) / SCAN_TILE;
  auto lay = [&](Carve& c) {
    h->ids = c.take<unsigned long long>(n);
    h->xy = c.take<float2>(n);
    h->radius = c.take<float>(n);
    h->cell = c.take<int2>(n);
    h->bucket = c.take<uint32_t>(n);
    h->rank = c.take<uint32_t>(n);
    h->sorted = c.take<uint32_t>(n);
    h->count = c.take<uint32_t>(nb);
    h->start = c.take<uint32_t>(nb + 1);
    h->tile_sums = c.take<uint32_t>(n_tiles);
    h->sub_bins = c.take<uint32_t>(COUNTER_BINS);
    h->status = c.take<uint32_t>(1);
  };
  Carve sizer;
  lay(sizer);
  e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = ensure(&h->pts, &h->pts_bytes, sizer.off + 256);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  Carve c;
  c.base = static_cast<char*>(h->pts);
  lay(c);
  h->n = (uint32_t)n;
  h->n_buckets = nb;
  if (n) {
    e = cudaMemcpyAsync(h->ids, ids, 8 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->xy, xy, 8 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->radius, radius, 4 * n, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(h->count, 0, 4 * (size_t)nb, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->status, 0, 4, st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  const HashDev d = h->dev();
  if (n) k_sh_keys<<<nblk(n), 256, 0, st>>>(d);
  scan_counts(h->count, h->start, nb, h->tile_sums, h->sub_bins, st);
  if (n) k_sh_scatter<<<nblk(n), 256, 0, st>>>(d, h->status);
  uint32_t status = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, h->status, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  return status ? BLOBS_ERR_INVALID_ARGUMENT : BLOBS_OK;
}

int blobs_spatial_hash_query(blobs_spatial_hash* h, uint64_t nq, const float* qxy, const float* qradius,
                             uint64_t* offsets, uint64_t* ids, uint64_t cap, uint64_t* total) {
  if (!h) return BLOBS_ERR_INVALID_HANDLE;
  if (!total || !offsets || (nq && (!qxy || !qradius)) || (cap && !ids)) return BLOBS_ERR_INVALID_ARGUMENT;
  if (nq > 0x3fffffffull) return BLOBS_ERR_INVALID_ARGUMENT;
  *total = 0;
  offsets[0] = 0;
  if (!nq) return BLOBS_OK;
  if (!h->pts) return BLOBS_ERR_STATE;
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  cudaStream_t st = h->stream;
  const uint32_t n_tiles = (uint32_t)((nq + SCAN_TILE - 1) / SCAN_TILE);
  float2* dq = nullptr;
  float* dr = nullptr;
  uint32_t *qcount = nullptr, *qstart = nullptr, *tiles = nullptr, *bins = nullptr;
  auto lay = [&](Carve& c) {
    dq = c.take<float2>(nq);
    dr = c.take<float>(nq);
    qcount = c.take<uint32_t>(nq);
    qstart = c.take<uint32_t>(nq + 1);
    tiles = c.take<uint32_t>(n_tiles);
    bins = c.take<uint32_t>(COUNTER_BINS);
  };
  Carve sizer;
  lay(sizer);
  e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = ensure(&h->qmem, &h->qmem_bytes, sizer.off + 256);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  Carve c;
  c.base = static_cast<char*>(h->qmem);
  lay(c);
  e = cudaMemcpyAsync(dq, qxy, 8 * nq, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dr, qradius, 4 * nq, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  const HashDev d = h->dev();
  k_sh_query<false><<<nblk(nq), 256, 0, st>>>(d, h->ids, (uint32_t)nq, dq, dr, qcount, nullptr, nullptr, 0ull);
  // totals above 2^32 - 1 would wrap the u32 scan: refused below
  scan_counts(qcount, qstart, (uint32_t)nq, tiles, bins, st);
  std::vector<uint32_t> hstart(nq + 1);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(hstart.data(), qstart, 4 * (nq + 1), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  uint64_t run = 0;
  for (uint64_t q = 0; q <= nq; ++q) {
    offsets[q] = hstart[q];
    if (q && hstart[q] < hstart[q - 1]) return BLOBS_ERR_OVERFLOW;  // the u32 prefix wrapped
    run = hstart[q];
  }
  *total = run;
  if (run > cap) return BLOBS_ERR_OVERFLOW;
  if (!run) return BLOBS_OK;
  e = ensure(&h->omem, &h->omem_bytes, 8 * run);
  if (e != cudaSuccess) return blobs_map_cuda(e);
  unsigned long long* dout = static_cast<unsigned long long*>(h->omem);
  k_sh_query<true><<<nblk(nq), 256, 0, st>>>(d, h->ids, (uint32_t)nq, dq, dr, nullptr, qstart, dout, run);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(ids, dout, 8 * run, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return blobs_map_cuda(e);
}

}  // extern "C"
