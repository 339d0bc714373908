// mesh_dev.cu -- device-side mesh set-up (meshdev.h): the octree built from
// a divider level by level, its 2:1 balance, leaves in Z order, the
// neighbour table and the ghost-update face tables, all on the GPU, so that
// admitting a mesh costs a few launches instead of host work proportional
// to its blocks.
//
// Reference: BCMOctree.cpp:23-41 (build by divider), 66-96 (build from a
// pedigree list), 248-262 (Z order), 277-364 (neighbour search), 423-478
// (NeighborInfo), BlockManager.cpp:63-114 (face lists); the host builder
// octree.cpp restates the same rules and the tests hold the two equal.
//
// Leaves are found by key: the Morton code of the leaf's corner at level 15
// (x bit i at 3i, y at 3i+1, z at 3i+2, so key order within a root is the
// reference's Z order) with the root index above it.  A set of leaves that
// partitions the root grid, sorted by key, answers "which leaf contains this
// point" by one binary search: the last leaf whose key is not above the
// point's.  Inactive regions are leaves too (flagged), so every point has
// its leaf.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "meshdev.h"
#include "octree_div.h"

namespace bcmg {
namespace {

using namespace bcmg_oct;

// ---- device buffers ----------------------------------------------------------
// Stream-ordered: allocated and freed on the set-up's stream (cudaMallocAsync /
// cudaFreeAsync), so that building a mesh never waits for work that other
// streams have queued (a served mesh is built while other requests solve).
thread_local cudaStream_t g_stream = nullptr;
struct StreamScope {
  cudaStream_t prev;
  explicit StreamScope(cudaStream_t s) : prev(g_stream) { g_stream = s; }
  ~StreamScope() { g_stream = prev; }
};

template <typename T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  ~Buf() { if (p) cudaFreeAsync(p, s); }
  cudaError_t alloc(size_t count) {
    if (p) { cudaFreeAsync(p, s); p = nullptr; }
    n = count;
    s = g_stream;
    return cudaMallocAsync(reinterpret_cast<void**>(&p), (count ? count : 1) * sizeof(T), s);
  }
  T* release() { T* q = p; p = nullptr; n = 0; return q; }
  void swap(Buf& o) { std::swap(p, o.p); std::swap(n, o.n); std::swap(s, o.s); }
};

template <typename T>
cudaError_t dev_new(T** p, size_t count, cudaStream_t st) {
  return cudaMallocAsync(reinterpret_cast<void**>(p), (count ? count : 1) * sizeof(T), st);
}

#define DEV_TRY(x)                              \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return e_;           \
  } while (0)

constexpr int kScanThreads = 256, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

// ---- exclusive scan of int ----------------------------------------------------
// Each CTA scans a tile of 1024 values (4 per thread, then the CTA's thread
// sums), writing the tile total to sums[tile]; the totals are scanned the
// same way (recursively) and added back.
__global__ void __launch_bounds__(kScanThreads) scan_tiles(int* __restrict__ a, int n,
                                                         int* __restrict__ sums) {
  __shared__ int ws[kScanThreads / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    v[q] = base + q < n ? a[base + q] : 0;
    s += v[q];
  }
  // inclusive scan of the thread sums: warp shuffles, then across warps
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < kScanThreads / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanThreads / 32) ws[lane] = t;
  }
  __syncthreads();
  int run = x - s + (w > 0 ? ws[w - 1] : 0);  // exclusive prefix of this thread
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    if (base + q < n) a[base + q] = run;
    run += v[q];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = run;
}

__global__ void scan_add(int* __restrict__ a, int n, const int* __restrict__ offs) {
  const int i = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
  for (int q = 0; q < kScanItems; q++)
    if (i + q < n) a[i + q] += offs[blockIdx.x];
}

// In place; *total (host) the sum of the inputs.
cudaError_t scan_excl(int* a, int n, int* total, cudaStream_t st) {
  if (n <= 0) {
    if (total) *total = 0;
    return cudaSuccess;
  }
  const int tiles = (n + kScanTile - 1) / kScanTile;
  Buf<int> sums;
  DEV_TRY(sums.alloc(tiles + 1));
  scan_tiles<<<tiles, kScanThreads, 0, st>>>(a, n, sums.p);
  DEV_TRY(cudaGetLastError());
  if (tiles > 1) {
    DEV_TRY(scan_excl(sums.p, tiles, total, st));
    scan_add<<<tiles, kScanThreads, 0, st>>>(a, n, sums.p);
    DEV_TRY(cudaGetLastError());
  } else if (total) {
    DEV_TRY(cudaMemcpyAsync(total, sums.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DEV_TRY(cudaStreamSynchronize(st));
  }
  return cudaSuccess;
}

// ---- stable radix sort of (uint64 key, int value) -----------------------------
// LSD, 8-bit digits, tiles of 1024 pairs per CTA.  Per pass: each tile's digit
// histogram (hist[digit * tiles + tile]); one exclusive scan over it gives
// every (digit, tile) its first output slot; each tile then places its pairs
// in order -- four groups of 256, a pair's rank among equal digits from the
// warp (match_any) and the earlier warps and groups (shared counters).
constexpr int kSortThreads = 256, kSortTile = 1024;

__global__ void __launch_bounds__(kSortThreads) sort_hist(const uint64_t* __restrict__ k, int n,
                                                        int shift, int* __restrict__ hist,
                                                        int tiles) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  for (int i = threadIdx.x; i < kSortTile; i += kSortThreads)
    if (base + i < n) atomicAdd(&h[(k[base + i] >> shift) & 255], 1);
  __syncthreads();
  hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) sort_scatter(
    const uint64_t* __restrict__ k, const int* __restrict__ v, int n, int shift,
    const int* __restrict__ hist, int tiles, uint64_t* __restrict__ ko, int* __restrict__ vo) {
  constexpr int NW = kSortThreads / 32;
  __shared__ int run[256];     // pairs of each digit placed by earlier groups
  __shared__ int wc[NW][256];  // count of each digit per warp in this group of 256
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  run[threadIdx.x] = hist[threadIdx.x * tiles + blockIdx.x];
  const int base = blockIdx.x * kSortTile;
  for (int r = 0; r < kSortTile / kSortThreads; r++) {
    for (int q = 0; q < NW; q++) wc[q][threadIdx.x] = 0;
    __syncthreads();
    const int i = base + r * kSortThreads + threadIdx.x;
    const bool ok = i < n;
    const int d = ok ? (int)((k[i] >> shift) & 255) : 256 + lane;  // unique dummy per lane
    const unsigned same = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(same & ((1u << lane) - 1));
    if (ok && rank == 0) wc[w][d] = __popc(same);
    __syncthreads();
    if (ok) {
      int before = run[d];
      for (int q = 0; q < w; q++) before += wc[q][d];
      ko[before + rank] = k[i];
      vo[before + rank] = v[i];
    }
    __syncthreads();
    int add = 0;
    for (int q = 0; q < NW; q++) add += wc[q][threadIdx.x];
    run[threadIdx.x] += add;
    __syncthreads();
  }
}

// Sorts (k, v) by the low `bits` bits of k, stably; the results end in k, v.
cudaError_t radix_sort(Buf<uint64_t>& k, Buf<int>& v, int n, int bits, cudaStream_t st) {
  if (n <= 1) return cudaSuccess;
  const int tiles = (n + kSortTile - 1) / kSortTile;
  Buf<uint64_t> k2;
  Buf<int> v2, hist;
  DEV_TRY(k2.alloc(n));
  DEV_TRY(v2.alloc(n));
  DEV_TRY(hist.alloc((size_t)256 * tiles));
  for (int shift = 0; shift < bits; shift += 8) {
    sort_hist<<<tiles, kSortThreads, 0, st>>>(k.p, n, shift, hist.p, tiles);
    DEV_TRY(cudaGetLastError());
    DEV_TRY(scan_excl(hist.p, 256 * tiles, nullptr, st));
    sort_scatter<<<tiles, kSortThreads, 0, st>>>(k.p, v.p, n, shift, hist.p, tiles, k2.p, v2.p);
    DEV_TRY(cudaGetLastError());
    k.swap(k2);
    v.swap(v2);
  }
  return cudaSuccess;
}

inline int blocks_for(int n, int t = 256) { return (n + t - 1) / t; }


// ---- face tables (BlockManager::setFaceLists, BlockManager.cpp:63-114) -------
enum : unsigned { FT_CONFLICT = 1, FT_NEUMANN = 2, FT_OPEN = 4, FT_PULL_BAD = 8 };

// Entries of face (b, f) per category: cnt[q * nbf + k], k = b*6+f, q = kind*3
// + axis; has[ax * nbf + k] = 1 when the face takes F2C entries.
__global__ void ft_count(int nb, const int* __restrict__ ld, const int* __restrict__ id,
                         const int* __restrict__ bctype, int* __restrict__ cnt,
                         int* __restrict__ has, unsigned* __restrict__ flags) {
  const int nbf = nb * 6, k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nbf) return;
  const int f = k % 6, ax = f / 2, l = ld[k];
  for (int q = 0; q < 12; q++) cnt[q * nbf + k] = 0;
  for (int a = 0; a < 3; a++) has[a * nbf + k] = 0;
  if (l == 0 || l == -1) {
    if (id[k * 4] >= 0) cnt[(l == 0 ? VC_COPY : VC_C2F) * 3 * nbf + ax * nbf + k] = 1;
  } else {
    int c = 0;
    for (int s = 0; s < 4; s++) c += id[k * 4 + s] >= 0;
    cnt[(VC_F2C * 3 + ax) * nbf + k] = c;
    has[ax * nbf + k] = c > 0;
  }
  if (bctype) {
    const bool neu = bctype[k] == BCMG_BC_NEUMANN;
    if (bctype[k] == BCMG_BC_DIRICHLET || neu) {
      cnt[(VC_DIRICHLET * 3 + ax) * nbf + k] = 1;
      if (id[k * 4] >= 0 || id[k * 4 + 1] >= 0 || id[k * 4 + 2] >= 0 || id[k * 4 + 3] >= 0)
        atomicOr(flags, FT_CONFLICT);
      if (neu) atomicOr(flags, FT_NEUMANN);
    }
  }
}

// The entries of face (b, f) at their scanned positions.
__global__ void ft_emit(int nb, const int* __restrict__ ld, const int* __restrict__ id,
                        const int* __restrict__ sf, const int* __restrict__ bctype, int bcform,
                        const int* __restrict__ pos, const int* __restrict__ slot,
                        VcTask* __restrict__ all) {
  const int nbf = nb * 6, k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nbf) return;
  const int b = k / 6, f = k % 6, ax = f / 2, l = ld[k];
  VcTask t{};
  t.dst = b;
  t.face = (uint8_t)f;
  t.slot = -1;
  if (l == 0 || l == -1) {
    if (id[k * 4] >= 0) {
      t.src = id[k * 4];
      t.kind = l == 0 ? VC_COPY : VC_C2F;
      t.subface = l == 0 ? 0 : (uint8_t)sf[k];
      all[pos[(t.kind * 3 + ax) * nbf + k]] = t;
    }
  } else {
    int at = pos[(VC_F2C * 3 + ax) * nbf + k];
    for (int s = 0; s < 4; s++) {
      if (id[k * 4 + s] < 0) continue;
      t.src = id[k * 4 + s];
      t.kind = VC_F2C;
      t.subface = (uint8_t)s;
      t.slot = slot[ax * nbf + k];
      all[at++] = t;
    }
  }
  if (bctype) {
    const bool neu = bctype[k] == BCMG_BC_NEUMANN;
    if (bctype[k] == BCMG_BC_DIRICHLET || neu) {
      VcTask d{};
      d.dst = b;
      d.src = -1;
      d.face = (uint8_t)f;
      d.kind = VC_DIRICHLET;  // boundary-condition ghosts of the face
      d.flags = neu ? kTaskNeumann : bcform == BCMG_DIRICHLET_BCX ? 1 : 0;
      d.slot = -1;
      all[pos[(VC_DIRICHLET * 3 + ax) * nbf + k]] = d;
    }
  }
}

__global__ void ft_cat_starts(const int* __restrict__ pos, int nbf, int* __restrict__ out) {
  const int q = threadIdx.x;
  if (q < 12) out[q] = pos[q * nbf];
}

// Source block of entry i (key) and its position (value), entries [lo, hi).
__global__ void ft_src_keys(const VcTask* __restrict__ all, int lo, int hi,
                            uint64_t* __restrict__ key, int* __restrict__ val,
                            int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (lo + i >= hi) return;
  const int s = all[lo + i].src;
  key[i] = (uint64_t)s;
  val[i] = lo + i;
  atomicAdd(&count[s], 1);
}

__global__ void ft_gather(const VcTask* __restrict__ all, const int* __restrict__ idx, int n,
                          VcTask* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = all[idx[i]];
}

__global__ void ft_facein_init(FaceIn* __restrict__ fin, int nbf) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nbf) fin[k] = FaceIn{{-1, -1, -1, -1}, -1, 0};
}

__global__ void ft_facein_fill(const VcTask* __restrict__ all, int n, FaceIn* __restrict__ fin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const VcTask t = all[i];
  FaceIn& fi = fin[t.dst * 6 + t.face];
  fi.kind = t.kind;
  if (t.kind == VC_F2C) {
    fi.src[t.subface] = t.src;
  } else {
    fi.src[0] = t.src;
    fi.sub = t.subface;
  }
}

// Per block: faces fed, the pull form's descriptor, open faces.
__global__ void ft_blocks(int nb, const FaceIn* __restrict__ fin, const int* __restrict__ slot,
                          const int* __restrict__ has, const int* __restrict__ optr,
                          const int* __restrict__ bctype, unsigned char* __restrict__ fed,
                          BlockInfo* __restrict__ bi, unsigned* __restrict__ flags) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int nbf = nb * 6;
  BlockInfo r;
  const int nout = optr[b + 1] - optr[b];
  if (nout > kMaxOutEntries) atomicOr(flags, FT_PULL_BAD);
  r.flags = min(nout, kMaxOutEntries) << BI_OUT_SHIFT;
  r.out_begin = optr[b];
  unsigned char fd = 0;
  bool open = false;
  for (int f = 0; f < 6; f++) {
    const int k = b * 6 + f;
    const FaceIn fi = fin[k];
    const int face_slot = has[(f / 2) * nbf + k] ? slot[(f / 2) * nbf + k] : -1;
    r.csrc[f] = fi.kind == VC_COPY ? fi.src[0] : fi.kind == VC_C2F ? fi.src[0] * 4 + fi.sub
                                                                    : face_slot;
    if (fi.kind >= 0) {
      r.flags |= (int)(BI_FED << f);
      fd |= (unsigned char)(1u << f);
    }
    if (fi.kind == VC_COPY) r.flags |= (int)(BI_COPY << f);
    if (fi.kind == VC_C2F) r.flags |= 1 << bi_c2f_bit(f);
    const bool dir = bctype && bctype[k] == BCMG_BC_DIRICHLET;
    if (dir) r.flags |= 1 << (BI_DIR_SHIFT + f);
    if (fi.kind < 0 && !dir) open = true;
  }
  bi[b] = r;
  fed[b] = fd;
  if (open) atomicOr(flags, FT_OPEN);
}

int bits_for(int n) {
  int b = 0;
  while (b < 31 && (1 << b) < n) b++;
  return (b + 7) / 8 * 8;
}

// Entries [lo, hi) of `all` grouped by source block, stably: the CSR offsets
// (ptr, nb+1, owned by the caller) and the entries (out).
cudaError_t by_source(const VcTask* all, int lo, int hi, int nb, Buf<int>& ptr,
                      Buf<VcTask>& out, cudaStream_t st) {
  const int n = hi - lo;
  DEV_TRY(ptr.alloc(nb + 1));
  DEV_TRY(cudaMemsetAsync(ptr.p, 0, (nb + 1) * sizeof(int), st));
  DEV_TRY(out.alloc(n));
  if (n > 0) {
    Buf<uint64_t> key;
    Buf<int> val;
    DEV_TRY(key.alloc(n));
    DEV_TRY(val.alloc(n));
    ft_src_keys<<<blocks_for(n), 256, 0, st>>>(all, lo, hi, key.p, val.p, ptr.p);
    DEV_TRY(cudaGetLastError());
    DEV_TRY(radix_sort(key, val, n, bits_for(nb), st));
    ft_gather<<<blocks_for(n), 256, 0, st>>>(all, val.p, n, out.p);
    DEV_TRY(cudaGetLastError());
  }
  return scan_excl(ptr.p, nb + 1, nullptr, st);
}

}  // namespace

cudaError_t build_face_tables(int nb, const int* ld, const int* id, const int* sf,
                              const int* bctype, int bcform, FaceTables* out,
                              cudaStream_t st) {
  StreamScope scope(st);
  const int nbf = nb * 6;
  Buf<int> pos, slot, starts;
  Buf<unsigned> flags;
  DEV_TRY(pos.alloc((size_t)12 * nbf));
  DEV_TRY(slot.alloc((size_t)3 * nbf));
  DEV_TRY(starts.alloc(12));
  DEV_TRY(flags.alloc(1));
  DEV_TRY(cudaMemsetAsync(flags.p, 0, sizeof(unsigned), st));
  ft_count<<<blocks_for(nbf), 256, 0, st>>>(nb, ld, id, bctype, pos.p, slot.p, flags.p);
  DEV_TRY(cudaGetLastError());
  // the face's has-F2C flags, before their scan turns them into slots
  Buf<int> has;
  DEV_TRY(has.alloc((size_t)3 * nbf));
  DEV_TRY(cudaMemcpyAsync(has.p, slot.p, (size_t)3 * nbf * sizeof(int), cudaMemcpyDeviceToDevice,
                          st));
  int ntasks = 0, slots = 0;
  DEV_TRY(scan_excl(pos.p, 12 * nbf, &ntasks, st));
  DEV_TRY(scan_excl(slot.p, 3 * nbf, &slots, st));
  ft_cat_starts<<<1, 32, 0, st>>>(pos.p, nbf, starts.p);
  DEV_TRY(cudaGetLastError());
  int cs[12];
  DEV_TRY(cudaMemcpyAsync(cs, starts.p, sizeof(cs), cudaMemcpyDeviceToHost, st));
  DEV_TRY(cudaStreamSynchronize(st));
  Buf<VcTask> all;
  DEV_TRY(all.alloc(ntasks));
  ft_emit<<<blocks_for(nbf), 256, 0, st>>>(nb, ld, id, sf, bctype, bcform, pos.p, slot.p, all.p);
  DEV_TRY(cudaGetLastError());
  const int nnd = cs[VC_DIRICHLET * 3];  // entries fed by neighbours come first
  Buf<int> pptr, optr;
  Buf<VcTask> push, outs;
  DEV_TRY(by_source(all.p, 0, nnd, nb, pptr, push, st));
  DEV_TRY(by_source(all.p, cs[VC_F2C * 3], cs[VC_C2F * 3], nb, optr, outs, st));
  Buf<FaceIn> fin;
  DEV_TRY(fin.alloc(nbf));
  ft_facein_init<<<blocks_for(nbf), 256, 0, st>>>(fin.p, nbf);
  if (nnd > 0) ft_facein_fill<<<blocks_for(nnd), 256, 0, st>>>(all.p, nnd, fin.p);
  Buf<unsigned char> fed;
  Buf<BlockInfo> bi;
  DEV_TRY(fed.alloc(nb));
  DEV_TRY(bi.alloc(nb));
  ft_blocks<<<blocks_for(nb), 256, 0, st>>>(nb, fin.p, slot.p, has.p, optr.p, bctype, fed.p, bi.p,
                                            flags.p);
  DEV_TRY(cudaGetLastError());
  unsigned hf = 0;
  DEV_TRY(cudaMemcpyAsync(&hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, st));
  DEV_TRY(cudaStreamSynchronize(st));
  for (int q = 0; q < 12; q++) {
    out->cat_start[q] = cs[q];
    out->cat_count[q] = (q < 11 ? cs[q + 1] : ntasks) - cs[q];
  }
  out->ntasks = ntasks;
  out->ghost_slots = slots;
  out->bc_conflict = (hf & FT_CONFLICT) != 0;
  out->has_neumann = (hf & FT_NEUMANN) != 0;
  out->open_faces = (hf & FT_OPEN) != 0;
  out->pull_ok = (hf & FT_PULL_BAD) == 0;
  out->tasks = ntasks ? all.release() : nullptr;
  out->push_ptr = pptr.release();
  out->push_tasks = nnd ? push.release() : nullptr;
  out->facein = fin.release();
  out->binfo = bi.release();
  out->fed = fed.release();
  out->out_tasks = outs.n ? outs.release() : nullptr;
  return cudaSuccess;
}


// ---- the octree on the device ---------------------------------------------------
namespace {

__host__ __device__ inline uint64_t spread3(unsigned v) {
  uint64_t x = v & 0x1fffffu;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}
// Key of a node: root index, then the Morton code of its corner at level 15.
__host__ __device__ inline uint64_t node_key(uint64_t p) {
  const unsigned sh = 15 - ped_level(p);
  return ((uint64_t)ped_root(p) << 45) | spread3(ped_x(p) << sh) | (spread3(ped_y(p) << sh) << 1) |
         (spread3(ped_z(p) << sh) << 2);
}
// Key and level together: distinct for distinct nodes (a node and its first
// descendants share a corner).
__host__ __device__ inline uint64_t node_key2(uint64_t p) { return (node_key(p) << 4) | ped_level(p); }

// Index of the last key not above q (the leaf containing point q when the
// sorted keys are those of a partition), -1 if none.
__device__ inline int find_leaf(const uint64_t* __restrict__ keys, int n, uint64_t q) {
  int lo = 0, hi = n;  // first index with key > q
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (keys[mid] <= q) lo = mid + 1;
    else hi = mid;
  }
  return lo - 1;
}
__device__ inline int find_exact(const uint64_t* __restrict__ keys, int n, uint64_t q) {
  const int i = find_leaf(keys, n, q);
  return i >= 0 && keys[i] == q ? i : -1;
}

// The same-level position across `face` (BCMOctree::findNeighborNode's
// target, BCMOctree.cpp:277-364): false across a non-periodic outer face.
__device__ inline bool across(const bcmg_rootgrid& rg, uint64_t p, int face, uint64_t* q) {
  const unsigned l = ped_level(p);
  long c[3] = {(long)ped_x(p), (long)ped_y(p), (long)ped_z(p)};
  const long mx = (1L << l) - 1;
  int r = (int)ped_root(p);
  const int ax = face / 2;
  c[ax] += (face % 2 == 0) ? -1 : 1;
  if (c[ax] < 0 || c[ax] > mx) {
    r = neighbor_root(rg, r, face);
    if (r < 0) return false;
    c[ax] = c[ax] < 0 ? mx : 0;
  }
  *q = ped_make(l, (unsigned)c[0], (unsigned)c[1], (unsigned)c[2], (unsigned)r);
  return true;
}

// ---- divider, level by level (BCMOctree::createTree) ----
__global__ void md_classify(const uint64_t* __restrict__ front, int n, bcmg_rootgrid rg,
                            bcmg_divider dv, int* __restrict__ nchild, int* __restrict__ nleaf,
                            unsigned char* __restrict__ cls) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t p = front[i];
  int c = divide(rg, dv, p);
  if (c == BRANCH && ped_level(p) >= 15) c = LEAF_ACTIVE;  // the deepest level stays a leaf
  cls[i] = (unsigned char)c;
  nchild[i] = c == BRANCH ? 8 : 0;
  nleaf[i] = c == BRANCH ? 0 : 1;
}

__global__ void md_expand(const uint64_t* __restrict__ front, int n,
                          const unsigned char* __restrict__ cls, const int* __restrict__ cpos,
                          const int* __restrict__ lpos, uint64_t* __restrict__ next,
                          uint64_t* __restrict__ lped, unsigned char* __restrict__ lact) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t p = front[i];
  if (cls[i] == BRANCH) {
    const unsigned l = ped_level(p) + 1;
    for (int c = 0; c < 8; c++)
      next[cpos[i] + c] = ped_make(l, ped_x(p) * 2 + (c & 1), ped_y(p) * 2 + ((c >> 1) & 1),
                                   ped_z(p) * 2 + ((c >> 2) & 1), ped_root(p));
  } else {
    lped[lpos[i]] = p;
    lact[lpos[i]] = cls[i] == LEAF_ACTIVE;
  }
}

__global__ void md_keys(const uint64_t* __restrict__ peds, int n, uint64_t* __restrict__ keys,
                        int* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = node_key(peds[i]);
  idx[i] = i;
}

template <typename T>
__global__ void md_permute(const T* __restrict__ in, const int* __restrict__ idx, int n,
                           T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[idx[i]];
}

// ---- 2:1 balance (a leaf two or more levels coarser than a face neighbour
// is refined, until none is) ----
__global__ void md_balance_mark(const uint64_t* __restrict__ keys,
                                const uint64_t* __restrict__ peds, int n, bcmg_rootgrid rg,
                                int* __restrict__ mark) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t p = peds[i];
  const unsigned l = ped_level(p);
  if (l < 2) return;
  for (int f = 0; f < 6; f++) {
    uint64_t q;
    if (!across(rg, p, f, &q)) continue;
    const int j = find_leaf(keys, n, node_key(q));
    if (j >= 0 && ped_level(peds[j]) + 1 < l) mark[j] = 1;
  }
}

__global__ void md_count_split(const int* __restrict__ mark, int n, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = mark[i] ? 8 : 1;
}

__global__ void md_split(const uint64_t* __restrict__ peds, const unsigned char* __restrict__ act,
                         const int* __restrict__ mark, const int* __restrict__ pos, int n,
                         uint64_t* __restrict__ op, unsigned char* __restrict__ oa,
                         uint64_t* __restrict__ ok) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t p = peds[i];
  if (!mark[i]) {
    op[pos[i]] = p;
    oa[pos[i]] = act[i];
    ok[pos[i]] = node_key(p);
    return;
  }
  const unsigned l = ped_level(p) + 1;
  for (int c = 0; c < 8; c++) {  // children in key order
    const uint64_t q = ped_make(l, ped_x(p) * 2 + (c & 1), ped_y(p) * 2 + ((c >> 1) & 1),
                                ped_z(p) * 2 + ((c >> 2) & 1), ped_root(p));
    op[pos[i] + c] = q;
    oa[pos[i] + c] = act[i];
    ok[pos[i] + c] = node_key(q);
  }
}

// ---- active leaves and their neighbour table ----
__global__ void md_flag(const unsigned char* __restrict__ act, int n, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = act[i];
}

__global__ void md_compact(const uint64_t* __restrict__ peds, const unsigned char* __restrict__ act,
                           const int* __restrict__ pos, int n, uint64_t* __restrict__ bped,
                           int* __restrict__ block_of) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  block_of[i] = act[i] ? pos[i] : -1;
  if (act[i]) bped[pos[i]] = peds[i];
}

// NeighborInfo of every block (BCMOctree.cpp:423-478, bcmg_octree_neighbors):
// the leaf at the same-level position across each face, its level
// difference, and for a subdivided position its four children on the face.
// `active`: the leaves the host tree holds active -- the blocks, and for a
// pedigree list also the roots it leaves untouched (a coarser such root
// still sets the level difference, with no neighbour id).
__global__ void md_neighbors(const uint64_t* __restrict__ keys, const uint64_t* __restrict__ peds,
                             const int* __restrict__ block_of,
                             const unsigned char* __restrict__ active, int n,
                             const uint64_t* __restrict__ bped, int nb, bcmg_rootgrid rg,
                             int* __restrict__ ld, int* __restrict__ id, int* __restrict__ sf,
                             int* __restrict__ outer, unsigned* __restrict__ err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb * 6) return;
  const int b = k / 6, f = k % 6;
  const uint64_t p = bped[b];
  const unsigned l = ped_level(p);
  int lv = 0, s0 = 0, ids[4] = {-1, -1, -1, -1};
  if (outer) outer[k] = on_outer(rg, p, f) ? 1 : 0;
  uint64_t q;
  if (across(rg, p, f, &q)) {
    const int j = find_leaf(keys, n, node_key(q));
    const unsigned lj = j >= 0 ? ped_level(peds[j]) : 0;
    if (j < 0) {
      atomicOr(err, 1u);  // not a partition
    } else if (lj + 1 == l) {
      if (active[j]) {
        lv = -1;
        ids[0] = block_of[j];
        s0 = child_to_subface(f, (int)ped_child_at(p, l));
      }
    } else if (lj == l) {
      ids[0] = block_of[j];
    } else if (lj > l) {
      lv = 1;
      for (int s = 0; s < 4; s++) {
        const int c = neighbor_child(f, s);
        const uint64_t cq = ped_make(l + 1, ped_x(q) * 2 + (c & 1), ped_y(q) * 2 + ((c >> 1) & 1),
                                     ped_z(q) * 2 + ((c >> 2) & 1), ped_root(q));
        const int jc = find_leaf(keys, n, node_key(cq));
        if (jc < 0 || ped_level(peds[jc]) != l + 1) {
          atomicOr(err, 2u);  // 2:1 broken across this face
          continue;
        }
        ids[s] = block_of[jc];
      }
    }
  }
  ld[k] = lv;
  sf[k] = s0;
  for (int s = 0; s < 4; s++) id[k * 4 + s] = ids[s];
}

// ---- completion of a pedigree list to a partition (BCMOctree.cpp:66-96: the
// siblings made on the way down to a listed leaf are inactive leaves) ----
__global__ void md_ancestor_count(const uint64_t* __restrict__ peds, int n, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = (int)ped_level(peds[i]);
}
__global__ void md_ancestors(const uint64_t* __restrict__ peds, int n, const int* __restrict__ pos,
                             uint64_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t p = peds[i];
  const unsigned l = ped_level(p);
  for (unsigned a = 0; a < l; a++) {
    const unsigned sh = l - a;
    out[pos[i] + a] = node_key2(ped_make(a, ped_x(p) >> sh, ped_y(p) >> sh, ped_z(p) >> sh,
                                         ped_root(p)));
  }
}
// 1 where a sorted key differs from its predecessor
__global__ void md_first(const uint64_t* __restrict__ k, int n, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i == 0 || k[i] != k[i - 1];
}
__global__ void md_unique(const uint64_t* __restrict__ k, const int* __restrict__ pos, int n,
                          uint64_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && (i == 0 || k[i] != k[i - 1])) out[pos[i]] = k[i];
}
// Key2 -> pedigree (the inverse of node_key2)
__device__ inline uint64_t ped_of_key2(uint64_t k2) {
  const unsigned l = (unsigned)(k2 & 0xf);
  const uint64_t key = k2 >> 4;
  unsigned c[3] = {0, 0, 0};
  for (int b = 0; b < 15; b++)
    for (int a = 0; a < 3; a++) c[a] |= (unsigned)((key >> (3 * b + a)) & 1) << b;
  const unsigned sh = 15 - l;
  return ped_make(l, c[0] >> sh, c[1] >> sh, c[2] >> sh, (unsigned)(key >> 45));
}
// Children of every ancestor, then every root: the candidate leaves.
__global__ void md_candidates(const uint64_t* __restrict__ anc, int na, int nroot,
                             uint64_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < na) {
    const uint64_t p = ped_of_key2(anc[i]);
    const unsigned l = ped_level(p) + 1;
    for (int c = 0; c < 8; c++)
      out[8 * i + c] = node_key2(ped_make(l, ped_x(p) * 2 + (c & 1), ped_y(p) * 2 + ((c >> 1) & 1),
                                          ped_z(p) * 2 + ((c >> 2) & 1), ped_root(p)));
  } else if (i < na + nroot) {
    out[8 * na + (i - na)] = node_key2(ped_make(0, 0, 0, 0, (unsigned)(i - na)));
  }
}
// Unique candidates that are no ancestor: the partition's leaves.
__global__ void md_leaf_flag(const uint64_t* __restrict__ cand, int n,
                             const uint64_t* __restrict__ anc, int na, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool first = i == 0 || cand[i] != cand[i - 1];
  flag[i] = first && find_exact(anc, na, cand[i]) < 0;
}
__global__ void md_leaf_emit(const uint64_t* __restrict__ cand, const int* __restrict__ flag,
                             const int* __restrict__ pos, int n, uint64_t* __restrict__ peds) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) peds[pos[i]] = ped_of_key2(cand[i]);
}
// The listed leaves among the partition's: active, block id = list index.
__global__ void md_mark_listed(const uint64_t* __restrict__ list, int n,
                               const uint64_t* __restrict__ keys,
                               const uint64_t* __restrict__ peds, int nl,
                               unsigned char* __restrict__ act, int* __restrict__ block_of,
                               unsigned* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = find_exact(keys, nl, node_key(list[i]));
  if (j < 0 || peds[j] != list[i]) {
    atomicOr(err, 4u);  // a listed leaf with listed leaves below it
    return;
  }
  if (atomicCAS(&block_of[j], -1, i) != -1) atomicOr(err, 8u);  // listed twice
  act[j] = 1;
}

__global__ void md_untouched_roots(const uint64_t* __restrict__ peds, int n,
                                   unsigned char* __restrict__ act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && ped_level(peds[i]) == 0) act[i] = 1;
}

__global__ void md_fill_int(int* __restrict__ a, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// ---- host side ----
// Leaves (peds, act) of a partition, any order: sorted by key.
cudaError_t sort_leaves(Buf<uint64_t>& peds, Buf<unsigned char>& act, Buf<uint64_t>& keys, int n,
                        int nroot, cudaStream_t st) {
  Buf<int> idx;
  DEV_TRY(keys.alloc(n));
  DEV_TRY(idx.alloc(n));
  if (n == 0) return cudaSuccess;
  md_keys<<<blocks_for(n), 256, 0, st>>>(peds.p, n, keys.p, idx.p);
  DEV_TRY(cudaGetLastError());
  int rb = 0;
  while ((1 << rb) < nroot) rb++;
  DEV_TRY(radix_sort(keys, idx, n, (45 + rb + 7) / 8 * 8, st));
  Buf<uint64_t> p2;
  Buf<unsigned char> a2;
  DEV_TRY(p2.alloc(n));
  DEV_TRY(a2.alloc(n));
  md_permute<<<blocks_for(n), 256, 0, st>>>(peds.p, idx.p, n, p2.p);
  md_permute<<<blocks_for(n), 256, 0, st>>>(act.p, idx.p, n, a2.p);
  DEV_TRY(cudaGetLastError());
  peds.swap(p2);
  act.swap(a2);
  return cudaSuccess;
}

// 2:1 balance of a sorted partition, in place (children replace their
// parents at its position, so the order stays the key order).
cudaError_t balance_leaves(Buf<uint64_t>& peds, Buf<unsigned char>& act, Buf<uint64_t>& keys,
                           int* n, const bcmg_rootgrid& rg, cudaStream_t st) {
  for (int pass = 0; pass < 64; pass++) {
    const int m = *n;
    Buf<int> mark, pos;
    DEV_TRY(mark.alloc(m));
    DEV_TRY(pos.alloc(m));
    DEV_TRY(cudaMemsetAsync(mark.p, 0, (size_t)m * sizeof(int), st));
    md_balance_mark<<<blocks_for(m), 256, 0, st>>>(keys.p, peds.p, m, rg, mark.p);
    md_count_split<<<blocks_for(m), 256, 0, st>>>(mark.p, m, pos.p);
    DEV_TRY(cudaGetLastError());
    int total = 0;
    DEV_TRY(scan_excl(pos.p, m, &total, st));
    if (total == m) return cudaSuccess;  // nothing marked
    Buf<uint64_t> p2, k2;
    Buf<unsigned char> a2;
    DEV_TRY(p2.alloc(total));
    DEV_TRY(k2.alloc(total));
    DEV_TRY(a2.alloc(total));
    md_split<<<blocks_for(m), 256, 0, st>>>(peds.p, act.p, mark.p, pos.p, m, p2.p, a2.p, k2.p);
    DEV_TRY(cudaGetLastError());
    peds.swap(p2);
    act.swap(a2);
    keys.swap(k2);
    *n = total;
  }
  return cudaErrorUnknown;  // a 15-level tree balances in fewer passes
}

// The neighbour table of blocks bped[nb] against the sorted partition.
int neighbors_of(const Buf<uint64_t>& keys, const Buf<uint64_t>& peds, const Buf<int>& block_of,
                 const Buf<unsigned char>& act, int n, MeshDev* m, const bcmg_rootgrid& rg,
                 cudaStream_t st, const char** why) {
  const int nb = m->nb;
  if (dev_new(&m->ld, (size_t)nb * 6, st) != cudaSuccess ||
      dev_new(&m->id, (size_t)nb * 24, st) != cudaSuccess ||
      dev_new(&m->sf, (size_t)nb * 6, st) != cudaSuccess ||
      dev_new(&m->outer, (size_t)nb * 6, st) != cudaSuccess) {
    *why = "device memory";
    return BCMG_MEMORY;
  }
  Buf<unsigned> err;
  if (err.alloc(1) != cudaSuccess) { *why = "device memory"; return BCMG_MEMORY; }
  cudaMemsetAsync(err.p, 0, sizeof(unsigned), st);
  md_neighbors<<<blocks_for(nb * 6), 256, 0, st>>>(keys.p, peds.p, block_of.p, act.p, n, m->peds, nb, rg,
                                                   m->ld, m->id, m->sf, m->outer, err.p);
  unsigned he = 0;
  if (cudaMemcpyAsync(&he, err.p, sizeof(he), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    *why = cudaGetErrorString(cudaGetLastError());
    return BCMG_CUDA_ERROR;
  }
  if (he & 2u) { *why = "level difference above one across a face (tree not 2:1 balanced)"; return BCMG_FAILURE; }
  if (he) { *why = "leaves do not partition the root grid"; return BCMG_FAILURE; }
  return BCMG_SUCCESS;
}

// Active leaves of a sorted partition in key order: pedigrees and block ids.
cudaError_t compact_active(const Buf<uint64_t>& peds, const Buf<unsigned char>& act, int n,
                           Buf<int>& block_of, MeshDev* m, cudaStream_t st) {
  Buf<int> pos;
  DEV_TRY(pos.alloc(n));
  DEV_TRY(block_of.alloc(n));
  md_flag<<<blocks_for(n), 256, 0, st>>>(act.p, n, pos.p);
  DEV_TRY(cudaGetLastError());
  int nb = 0;
  DEV_TRY(scan_excl(pos.p, n, &nb, st));
  m->nb = nb;
  DEV_TRY(dev_new(&m->peds, (size_t)nb, st));
  md_compact<<<blocks_for(n), 256, 0, st>>>(peds.p, act.p, pos.p, n, m->peds, block_of.p);
  return cudaGetLastError();
}

// The partition that a leaf list makes (listed leaves, siblings of their
// ancestors, untouched roots), sorted by key, with its block ids and
// active flags (the listed leaves).
int complete_list(const bcmg_rootgrid& rg, const Buf<uint64_t>& list, int n, Buf<uint64_t>& peds,
                  Buf<unsigned char>& act, Buf<uint64_t>& keys, Buf<int>& block_of, int* nl,
                  cudaStream_t st, const char** why) {
  const int nroot = rg_nroot(rg);
  int rb = 0;
  while ((1 << rb) < nroot) rb++;
  const int kbits = (45 + rb + 4 + 7) / 8 * 8;
  Buf<int> cnt, idx;
  if (cnt.alloc(n) != cudaSuccess) return BCMG_MEMORY;
  int na_all = 0;
  md_ancestor_count<<<blocks_for(n), 256, 0, st>>>(list.p, n, cnt.p);
  if (scan_excl(cnt.p, n, &na_all, st) != cudaSuccess) return BCMG_CUDA_ERROR;
  Buf<uint64_t> anc, ancu;
  if (anc.alloc(na_all) != cudaSuccess || idx.alloc(na_all) != cudaSuccess) return BCMG_MEMORY;
  md_ancestors<<<blocks_for(n), 256, 0, st>>>(list.p, n, cnt.p, anc.p);
  if (na_all) md_fill_int<<<blocks_for(na_all), 256, 0, st>>>(idx.p, na_all, 0);
  if (radix_sort(anc, idx, na_all, kbits, st) != cudaSuccess) return BCMG_CUDA_ERROR;
  // unique ancestors
  int na = 0;
  {
    Buf<int> pos;
    if (pos.alloc(na_all) != cudaSuccess || ancu.alloc(na_all) != cudaSuccess) return BCMG_MEMORY;
    if (na_all) md_first<<<blocks_for(na_all), 256, 0, st>>>(anc.p, na_all, pos.p);
    if (scan_excl(pos.p, na_all, &na, st) != cudaSuccess) return BCMG_CUDA_ERROR;
    if (na_all) md_unique<<<blocks_for(na_all), 256, 0, st>>>(anc.p, pos.p, na_all, ancu.p);
  }
  // candidates: children of the ancestors and the roots
  const int nc = 8 * na + nroot;
  Buf<uint64_t> cand;
  Buf<int> cidx, flag, pos;
  if (cand.alloc(nc) != cudaSuccess || cidx.alloc(nc) != cudaSuccess ||
      flag.alloc(nc) != cudaSuccess || pos.alloc(nc) != cudaSuccess)
    return BCMG_MEMORY;
  md_candidates<<<blocks_for(na + nroot), 256, 0, st>>>(ancu.p, na, nroot, cand.p);
  md_fill_int<<<blocks_for(nc), 256, 0, st>>>(cidx.p, nc, 0);
  if (radix_sort(cand, cidx, nc, kbits, st) != cudaSuccess) return BCMG_CUDA_ERROR;
  md_leaf_flag<<<blocks_for(nc), 256, 0, st>>>(cand.p, nc, ancu.p, na, flag.p);
  if (cudaMemcpyAsync(pos.p, flag.p, (size_t)nc * sizeof(int), cudaMemcpyDeviceToDevice, st) !=
      cudaSuccess)
    return BCMG_CUDA_ERROR;
  int m = 0;
  if (scan_excl(pos.p, nc, &m, st) != cudaSuccess) return BCMG_CUDA_ERROR;
  if (peds.alloc(m) != cudaSuccess || act.alloc(m) != cudaSuccess ||
      keys.alloc(m) != cudaSuccess || block_of.alloc(m) != cudaSuccess)
    return BCMG_MEMORY;
  md_leaf_emit<<<blocks_for(nc), 256, 0, st>>>(cand.p, flag.p, pos.p, nc, peds.p);
  {
    Buf<int> ki;
    if (ki.alloc(m) != cudaSuccess) return BCMG_MEMORY;
    md_keys<<<blocks_for(m), 256, 0, st>>>(peds.p, m, keys.p, ki.p);  // already in key order
  }
  cudaMemsetAsync(act.p, 0, (size_t)m, st);
  md_fill_int<<<blocks_for(m), 256, 0, st>>>(block_of.p, m, -1);
  Buf<unsigned> err;
  if (err.alloc(1) != cudaSuccess) return BCMG_MEMORY;
  cudaMemsetAsync(err.p, 0, sizeof(unsigned), st);
  md_mark_listed<<<blocks_for(n), 256, 0, st>>>(list.p, n, keys.p, peds.p, m, act.p, block_of.p,
                                                err.p);
  unsigned he = 0;
  if (cudaMemcpyAsync(&he, err.p, sizeof(he), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BCMG_CUDA_ERROR;
  if (he & 8u) { *why = "a leaf is listed twice"; return BCMG_USAGE; }
  if (he) { *why = "a listed leaf has listed leaves below it"; return BCMG_USAGE; }
  *nl = m;
  return BCMG_SUCCESS;
}

}  // namespace

void mesh_free(MeshDev* m, cudaStream_t st) {
  if (m->peds) cudaFreeAsync(m->peds, st);
  if (m->ld) cudaFreeAsync(m->ld, st);
  if (m->id) cudaFreeAsync(m->id, st);
  if (m->sf) cudaFreeAsync(m->sf, st);
  if (m->outer) cudaFreeAsync(m->outer, st);
  *m = MeshDev{};
}

int mesh_from_divider(const bcmg_rootgrid& rg, const bcmg_divider& div, MeshDev* out,
                      cudaStream_t st, const char** why) {
  StreamScope scope(st);
  const int nroot = rg_nroot(rg);
  bcmg_divider dv = div;
  Buf<double> pts;
  if (dv.kind == BCMG_DIV_BALLS && dv.npoints > 0) {
    if (pts.alloc((size_t)dv.npoints * 3) != cudaSuccess) return BCMG_MEMORY;
    cudaMemcpyAsync(pts.p, div.points, (size_t)dv.npoints * 3 * sizeof(double),
                    cudaMemcpyHostToDevice, st);
    dv.points = pts.p;
  } else {
    dv.points = nullptr;
  }
  // level by level: the frontier of nodes still to decide, and the leaves
  std::vector<uint64_t> roots(nroot);
  for (int r = 0; r < nroot; r++) roots[r] = ped_make(0, 0, 0, 0, (unsigned)r);
  Buf<uint64_t> front, lped;
  Buf<unsigned char> lact;
  if (front.alloc(nroot) != cudaSuccess) return BCMG_MEMORY;
  cudaMemcpyAsync(front.p, roots.data(), (size_t)nroot * sizeof(uint64_t), cudaMemcpyHostToDevice,
                  st);
  int nf = nroot, nleaves = 0;
  Buf<uint64_t> allp;
  Buf<unsigned char> alla;
  struct Level { Buf<uint64_t> p; Buf<unsigned char> a; int n = 0; };  // leaves found per level
  std::vector<Level*> levels;
  int rc = BCMG_SUCCESS;
  while (nf > 0 && rc == BCMG_SUCCESS) {
    Buf<int> nchild, nleaf;
    Buf<unsigned char> cls;
    if (nchild.alloc(nf) != cudaSuccess || nleaf.alloc(nf) != cudaSuccess ||
        cls.alloc(nf) != cudaSuccess) { rc = BCMG_MEMORY; break; }
    md_classify<<<blocks_for(nf), 256, 0, st>>>(front.p, nf, rg, dv, nchild.p, nleaf.p, cls.p);
    int nnext = 0, nl = 0;
    if (scan_excl(nchild.p, nf, &nnext, st) != cudaSuccess ||
        scan_excl(nleaf.p, nf, &nl, st) != cudaSuccess) { rc = BCMG_CUDA_ERROR; break; }
    Level* lv = new Level;
    levels.push_back(lv);
    Buf<uint64_t> next;
    if (next.alloc(nnext) != cudaSuccess || lv->p.alloc(nl) != cudaSuccess ||
        lv->a.alloc(nl) != cudaSuccess) { rc = BCMG_MEMORY; break; }
    lv->n = nl;
    md_expand<<<blocks_for(nf), 256, 0, st>>>(front.p, nf, cls.p, nchild.p, nleaf.p, next.p,
                                              lv->p.p, lv->a.p);
    if (cudaGetLastError() != cudaSuccess) { rc = BCMG_CUDA_ERROR; break; }
    nleaves += nl;
    front.swap(next);
    nf = nnext;
  }
  if (rc == BCMG_SUCCESS) {
    if (allp.alloc(nleaves) != cudaSuccess || alla.alloc(nleaves) != cudaSuccess) rc = BCMG_MEMORY;
    int at = 0;
    for (Level* lv : levels) {
      if (rc == BCMG_SUCCESS && lv->n) {
        cudaMemcpyAsync(allp.p + at, lv->p.p, (size_t)lv->n * sizeof(uint64_t),
                        cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(alla.p + at, lv->a.p, (size_t)lv->n, cudaMemcpyDeviceToDevice, st);
        at += lv->n;
      }
    }
  }
  for (Level* lv : levels) delete lv;  // (frees after the copies: cudaFree synchronises)
  if (rc != BCMG_SUCCESS) { *why = "device memory"; return rc; }
  Buf<uint64_t> keys;
  int n = nleaves;
  if (sort_leaves(allp, alla, keys, n, nroot, st) != cudaSuccess) return BCMG_CUDA_ERROR;
  if (div.balance && balance_leaves(allp, alla, keys, &n, rg, st) != cudaSuccess)
    return BCMG_CUDA_ERROR;
  Buf<int> block_of;
  *out = MeshDev{};
  if (compact_active(allp, alla, n, block_of, out, st) != cudaSuccess) {
    mesh_free(out, st);
    return BCMG_CUDA_ERROR;
  }
  rc = out->nb > 0 ? neighbors_of(keys, allp, block_of, alla, n, out, rg, st, why) : BCMG_SUCCESS;
  if (rc != BCMG_SUCCESS) mesh_free(out, st);
  return rc;
}

int mesh_from_pedigrees(const bcmg_rootgrid& rg, const uint64_t* peds, int n, bool balance,
                        MeshDev* out, cudaStream_t st, const char** why) {
  StreamScope scope(st);
  const int nroot = rg_nroot(rg);
  if (n <= 0) { *why = "no leaves"; return BCMG_USAGE; }
  for (int i = 0; i < n; i++)
    if ((int)ped_root(peds[i]) >= nroot) { *why = "root index out of the root grid"; return BCMG_USAGE; }
  Buf<uint64_t> list, lp, keys;
  Buf<unsigned char> act;
  Buf<int> block_of;
  if (list.alloc(n) != cudaSuccess) return BCMG_MEMORY;
  cudaMemcpyAsync(list.p, peds, (size_t)n * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
  int m = 0;
  int rc = complete_list(rg, list, n, lp, act, keys, block_of, &m, st, why);
  if (rc != BCMG_SUCCESS) return rc;
  *out = MeshDev{};
  if (balance) {
    if (balance_leaves(lp, act, keys, &m, rg, st) != cudaSuccess ||
        compact_active(lp, act, m, block_of, out, st) != cudaSuccess) {
      mesh_free(out, st);
      return BCMG_CUDA_ERROR;
    }
  } else {
    out->nb = n;
    if (dev_new(&out->peds, (size_t)n, st) != cudaSuccess) return BCMG_MEMORY;
    cudaMemcpyAsync(out->peds, list.p, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
    // the host tree keeps the roots the list leaves untouched as active leaves
    md_untouched_roots<<<blocks_for(m), 256, 0, st>>>(lp.p, m, act.p);
  }
  rc = out->nb > 0 ? neighbors_of(keys, lp, block_of, act, m, out, rg, st, why) : BCMG_SUCCESS;
  if (rc != BCMG_SUCCESS) mesh_free(out, st);
  return rc;
}

}  // namespace bcmg
