// capi.cu -- the C ABI of include/bcmg.h: context, field arena, device face
// table and solver drivers.  Host code; all arithmetic runs in the kernels of
// vc.cu and stencil.cu.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <limits>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "bcmg.h"
#include "common.cuh"
#include "kernels.h"
#include "meshdev.h"
#include "stream.cuh"

using namespace bcmg;

namespace {

struct Field {
  int dtype = 0, vc = 0;
  void* d = nullptr;
  int64_t bstride = 0, brick = 0;
  size_t bytes = 0;
  int vc_method = -1;
  cudaEvent_t ev = nullptr;
  bool host = false;  // page-locked host memory mapped into the device's address space
};

struct OpRec {
  double* d_cc = nullptr;
  // fused Jacobi constants per block: {Ap, Aw, Ae, As, An, Ab, At, 1/Ap}
  float* d_jc32 = nullptr;
  double* d_jc64 = nullptr;
  int fields[7] = {-1, -1, -1, -1, -1, -1, -1};
};

size_t dsize(int dtype) { return dtype == BCMG_F64 ? 8 : 4; }

struct GraphKey {
  void *x, *b, *w;
  int op, iters;
  double omega;
  int choice;  // fused-Jacobi kernel choice
  bool operator<(const GraphKey& o) const {
    if (x != o.x) return x < o.x;
    if (b != o.b) return b < o.b;
    if (w != o.w) return w < o.w;
    if (op != o.op) return op < o.op;
    if (iters != o.iters) return iters < o.iters;
    if (choice != o.choice) return choice < o.choice;
    return omega < o.omega;
  }
};

struct GraphRec {
  cudaGraphExec_t exec;
  int64_t kernels;  // kernel launches one replay performs
};

}  // namespace

struct bcmg_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  // registered blocks
  int nb = 0, nx = 0, ny = 0, nz = 0;
  bool registered = false;
  std::vector<int> ld, id, sf;
  // meshes registered from the device set-up: leaf pedigrees and outer faces
  std::vector<uint64_t> peds;
  std::vector<int> outer;
  std::vector<void*> retired;  // replaced face tables, freed with the context

  // boundary
  std::vector<int> bctype;
  bool open_faces = true;  // some face has neither a neighbour nor a Dirichlet condition
  bool has_neumann = false;  // some face carries a Neumann condition (separate launches only)
  std::vector<double> bcval;
  int bcform = BCMG_DIRICHLET_SOR;
  int* d_bctype = nullptr;
  double* d_bcval = nullptr;
  double* d_bczero = nullptr;
  float* d_bcv2f = nullptr;    // [nb*8] 2v as an exact float, or NaN (BlockBc::v2f)
  float* d_bczero2f = nullptr; // the same for homogeneous values (zeros)
  bool bc_conflict = false;

  // face table, grouped into 12 categories: kind * 3 + axis
  VcTask* d_tasks = nullptr;
  int cat_start[12] = {}, cat_count[12] = {};
  int* d_push_ptr = nullptr;       // [nb+1] CSR of entries by source block
  VcTask* d_push_tasks = nullptr;
  unsigned char* d_fed = nullptr;  // [nb] faces fed by a neighbour
  FaceIn* d_facein = nullptr;      // [nb*6] ghost sources per face (pull form)
  BlockInfo* d_binfo = nullptr;    // [nb] block descriptors (pipelined pull form)
  VcTask* d_out_tasks = nullptr;   // F2C entries by source block (pull form)
  int ghost_slots = 0;             // side-buffer slots (faces across a level change)
  bool pull_ok = true;             // every block feeds at most kMaxOutEntries of them
  void* d_side[2] = {nullptr, nullptr};  // side buffers of first-layer ghosts
  size_t side_bytes = 0;
  size_t side_es = 0;                    // element size the side buffers are laid out for
  int ghost_form = BCMG_GHOST_AUTO;  // bcmg_set_ghost_form
  int jacobi_shape = 0;              // bcmg_set_jacobi_shape (0: automatic)
  int jacobi_force = 0;              // autotuner: the fused-Jacobi choice under test
  std::map<long, int> jacobi_tuned;  // tuned fused-Jacobi choice per (dtype, n, vc)

  std::map<int, Field> fields;
  int next_field = 1;
  std::map<int, OpRec> ops;
  int next_op = 1;
  std::map<long, int> work;  // cached solver work fields: key (dtype, vc, slot)

  double* d_partial = nullptr;
  double* d_scalar = nullptr;
  // device-resident BiCGSTAB: two partial sums per block, the segments'
  // scalar records and their pinned host mirror
  double* d_kpart = nullptr;
  KSeg* d_kseg = nullptr;
  KSeg* h_kseg = nullptr;
  int kseg_cap = 0;
  int kpart_nb = 0;
  // independent systems in one mesh (bcmg_set_segments): blocks
  // [seg_first[s], seg_first[s+1]) are segment s; one segment by default
  int nseg = 1;
  std::vector<int> seg_first;
  int* d_seg_of = nullptr;
  int* d_seg_first = nullptr;
  // per-segment arguments of the segmented kernels (flags, scales, limits)
  // and the segments' pairs of sums, device and pinned host copies
  unsigned char* d_segflag = nullptr;
  double* d_segscale = nullptr;
  int* d_segmaxit = nullptr;
  double* d_segeps2 = nullptr;
  double* d_segsum = nullptr;
  double* h_segsum = nullptr;
  int segbuf_cap = 0;
  int* d_err = nullptr;  // device error word: bounded waits that timed out
  double* h_scalar = nullptr;

  size_t budget = 0, in_use = 0;
  int64_t launches = 0;
  bool no_fusion = false;  // bcmg_set_fusion(0): separate sweep + gather launches
  int sor_fixed = 0;       // bcmg_set_sor_variant: forced SOR kernel shape (0 = auto)
  std::map<long, int> sor_tuned;  // autotuned shape per (dtype, n, vc, form)
  std::map<GraphKey, GraphRec> graphs;  // captured Jacobi runs (bcmg_jacobi_run)

  // optional per-launch CUDA-event timing (bcmg_profile_*)
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;     // kernel kind of each recorded pair
  size_t ev_used = 0;           // events in use (pairs * 2)
};

// ---------------------------------------------------------------------------
static int fail(bcmg_ctx c, int code, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}

#define CUDA_TRY(c, expr)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail((c), BCMG_CUDA_ERROR, "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_),   \
                  __FILE__, __LINE__);                                                     \
  } while (0)

// Kernel kinds for bcmg_profile_kernel.
enum { K_VC = 0, K_SOR = 1, K_JACOBI = 2, K_RESIDUAL = 3, K_DOT = 4, K_BLAS1 = 5, K_FILL = 6,
       K_OTHER = 7, K_NKINDS = 8 };

static void prof_mark(bcmg_ctx c, int kind, cudaStream_t st, bool start);

#define LAUNCH(c, kind, st, expr)                                                          \
  do {                                                                                     \
    prof_mark((c), (kind), (st), true);                                                    \
    cudaError_t e_ = (expr);                                                               \
    prof_mark((c), (kind), (st), false);                                                   \
    (c)->launches++;                                                                       \
    if (e_ != cudaSuccess)                                                                 \
      return fail((c), BCMG_CUDA_ERROR, "launch failed: %s (%s:%d)", cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                     \
  } while (0)

static void prof_mark(bcmg_ctx c, int kind, cudaStream_t st, bool start) {
  if (!c->profiling) return;
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); c->profiling = false; return; }
    c->ev_pool.push_back(e);
  }
  if (start) c->ev_kind.push_back(kind);
  cudaEventRecord(c->ev_pool[c->ev_used++], st);
}

static cudaStream_t S(bcmg_ctx c, void* st) { return st ? (cudaStream_t)st : c->stream; }

static Field* get_field(bcmg_ctx c, int f) {
  auto it = c->fields.find(f);
  return it == c->fields.end() ? nullptr : &it->second;
}

static Geom geom_of(bcmg_ctx c, const Field& f) {
  Geom g;
  g.nx = c->nx; g.ny = c->ny; g.nz = c->nz; g.vc = f.vc;
  const int nx0 = c->nx + 2 * f.vc, ny0 = c->ny + 2 * f.vc;
  g.sy = nx0; g.sz = nx0 * ny0;
  g.off0 = (1 + nx0 + nx0 * ny0) * f.vc;
  g.bstride = f.bstride;
  g.nb = c->nb;
  return g;
}

static int dev_alloc(bcmg_ctx c, void** p, size_t bytes) {
  if (c->budget && c->in_use + bytes > c->budget)
    return fail(c, BCMG_MEMORY, "allocation of %zu bytes exceeds the memory budget (%zu of %zu in use)",
                bytes, c->in_use, c->budget);
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, BCMG_MEMORY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  c->in_use += bytes;
  return BCMG_SUCCESS;
}

static void dev_free(bcmg_ctx c, void* p, size_t bytes) {
  if (!p) return;
  cudaFree(p);
  c->in_use -= bytes;
}

// Device face table: the reference's local face list (BlockManager::setFaceLists,
// BlockManager.cpp:477-510) plus one entry per Dirichlet outer face.
static void clear_graphs(bcmg_ctx c);

// The face tables of the registered blocks, built on the device
// (build_face_tables, mesh_dev.cu) from the neighbour table and the faces'
// boundary types.
static int build_face_table(bcmg_ctx c) {
  // captured Jacobi runs hold the addresses of the tables rebuilt below
  cudaStreamSynchronize(c->stream);
  clear_graphs(c);
  const size_t nbf = (size_t)c->nb * 6;
  cudaStream_t st = c->stream;
  int *d_ld = nullptr, *d_id = nullptr, *d_sf = nullptr, *d_bt = nullptr;
  // stream-ordered, like the builder's own buffers: no wait for other streams
  auto release = [&] {
    for (int* q : {d_ld, d_id, d_sf, d_bt})
      if (q) cudaFreeAsync(q, st);
  };
  if (cudaMallocAsync(reinterpret_cast<void**>(&d_ld), nbf * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync(reinterpret_cast<void**>(&d_id), nbf * 4 * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync(reinterpret_cast<void**>(&d_sf), nbf * sizeof(int), st) != cudaSuccess ||
      (!c->bctype.empty() &&
       cudaMallocAsync(reinterpret_cast<void**>(&d_bt), nbf * sizeof(int), st) != cudaSuccess)) {
    release();
    return fail(c, BCMG_MEMORY, "face tables: device memory");
  }
  cudaMemcpyAsync(d_ld, c->ld.data(), nbf * sizeof(int), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_id, c->id.data(), nbf * 4 * sizeof(int), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_sf, c->sf.data(), nbf * sizeof(int), cudaMemcpyHostToDevice, st);
  if (d_bt) cudaMemcpyAsync(d_bt, c->bctype.data(), nbf * sizeof(int), cudaMemcpyHostToDevice, st);
  FaceTables ft;
  const cudaError_t e = build_face_tables(c->nb, d_ld, d_id, d_sf, d_bt, c->bcform, &ft, st);
  release();
  if (e != cudaSuccess) return fail(c, BCMG_CUDA_ERROR, "face tables: %s", cudaGetErrorString(e));
  // the tables being replaced may still be read by work on other streams:
  // they are freed with the context
  for (void* q : {(void*)c->d_tasks, (void*)c->d_push_ptr, (void*)c->d_push_tasks,
                  (void*)c->d_facein, (void*)c->d_binfo, (void*)c->d_fed, (void*)c->d_out_tasks})
    if (q) c->retired.push_back(q);
  c->d_tasks = ft.tasks;
  for (int q = 0; q < 12; q++) {
    c->cat_start[q] = ft.cat_start[q];
    c->cat_count[q] = ft.cat_count[q];
  }
  c->d_push_ptr = ft.push_ptr;
  c->d_push_tasks = ft.push_tasks;
  c->d_facein = ft.facein;
  c->d_binfo = ft.binfo;
  c->d_fed = ft.fed;
  c->d_out_tasks = ft.out_tasks;
  c->ghost_slots = ft.ghost_slots;
  c->pull_ok = ft.pull_ok;
  c->open_faces = ft.open_faces;
  c->bc_conflict = ft.bc_conflict;
  c->has_neumann = ft.has_neumann;
  return BCMG_SUCCESS;
}

// Slices of the face table for one launch.  ld bit (ld+1): C2F kind for ld=-1,
// COPY for 0, F2C for +1.
static VcRanges select_ranges(bcmg_ctx c, int axis_mask, int ld_mask, bool vc, bool bc) {
  VcRanges r{};
  r.n = 0;
  r.prefix[0] = 0;
  const int kind_of_ldbit[3] = {VC_C2F, VC_COPY, VC_F2C};
  auto add = [&](int q) {
    if (c->cat_count[q] == 0) return;
    r.start[r.n] = c->cat_start[q];
    r.prefix[r.n + 1] = r.prefix[r.n] + c->cat_count[q];
    r.n++;
  };
  // F2C first, then same level, then C2F (the SeparateLevelDiff order,
  // LocalScalar3D.h:214-224); the order is immaterial on one rank.
  const int ldbits[3] = {2, 1, 0};
  if (vc)
    for (int li = 0; li < 3; li++) {
      const int lb = ldbits[li];
      if (!((ld_mask >> lb) & 1)) continue;
      for (int ax = 0; ax < 3; ax++)
        if ((axis_mask >> ax) & 1) add(kind_of_ldbit[lb] * 3 + ax);
    }
  if (bc)
    for (int ax = 0; ax < 3; ax++) add(VC_DIRICHLET * 3 + ax);
  return r;
}

static int gather(bcmg_ctx c, Field& f, const VcRanges& r, bool homogeneous, cudaStream_t st) {
  if (r.n == 0) return BCMG_SUCCESS;
  Geom g = geom_of(c, f);
  VcTable tab{c->d_tasks, 0, homogeneous ? c->d_bczero : c->d_bcval};
  if (f.dtype == BCMG_F64)
    LAUNCH(c, K_VC, st, launch_vc_gather<double>((double*)f.d, g, tab, r, st));
  else
    LAUNCH(c, K_VC, st, launch_vc_gather<float>((float*)f.d, g, tab, r, st));
  return BCMG_SUCCESS;
}

// Drops every captured Jacobi run (they hold device addresses).
static void clear_graphs(bcmg_ctx c) {
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second.exec);
  c->graphs.clear();
}

// Side buffers of the pull form: the first ghost layer of every face across a
// level change, then the two x-face layers of every block (the pipelined
// kernels read same-level x ghosts from there: one coalesced row instead of
// one 32-byte sector per cell); one pair (input, output) per context, sized
// for the largest element type used so far.
static size_t side_elems(bcmg_ctx c) {
  return ((size_t)c->ghost_slots + 2 * (size_t)c->nb) * c->nx * c->ny;
}
static int ensure_side(bcmg_ctx c, size_t es) {
  const size_t need = std::max<size_t>(256, side_elems(c) * es);
  if (c->side_bytes >= need) {
    c->side_es = std::max(c->side_es, es);
    return BCMG_SUCCESS;
  }
  // captured runs hold the old buffers' addresses
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  clear_graphs(c);
  for (int k = 0; k < 2; k++) {
    cudaFree(c->d_side[k]);
    c->d_side[k] = nullptr;
  }
  c->side_bytes = 0;
  for (int k = 0; k < 2; k++) CUDA_TRY(c, cudaMalloc(&c->d_side[k], need));
  c->side_bytes = need;
  c->side_es = es;
  return BCMG_SUCCESS;
}

// Tables of a fused launch; `seq` counts the launches of a pull-form run
// (its side buffers alternate).
static PushTable push_table(bcmg_ctx c, int seq) {
  // x-face layers after the level-change slots, at the element size the
  // buffers were last sized for (one context runs one element size at a time)
  const size_t xo = (size_t)c->ghost_slots * c->nx * c->ny * c->side_es;
  unsigned char* s0 = static_cast<unsigned char*>(c->d_side[seq & 1]);
  unsigned char* s1 = static_cast<unsigned char*>(c->d_side[(seq + 1) & 1]);
  return PushTable{c->d_push_ptr, c->d_push_tasks, c->d_fed, c->d_facein, c->d_binfo,
                   c->d_out_tasks, s0, s1, s0 ? s0 + xo : nullptr, s1 ? s1 + xo : nullptr};
}

// ImposeBoundaryCondition: VC update of all faces, then Dirichlet ghosts.
static int impose(bcmg_ctx c, Field& f, bool homogeneous, cudaStream_t st) {
  if (!c->bc_conflict) return gather(c, f, select_ranges(c, 7, 7, true, true), homogeneous, st);
  int rc = gather(c, f, select_ranges(c, 7, 7, true, false), homogeneous, st);
  if (rc) return rc;
  return gather(c, f, select_ranges(c, 7, 7, false, true), homogeneous, st);
}

static int create_field(bcmg_ctx c, int dtype, int vc, int* out, bool host = false) {
  if (!c->registered) return fail(c, BCMG_USAGE, "no blocks registered");
  if (dtype != BCMG_F32 && dtype != BCMG_F64) return fail(c, BCMG_USAGE, "bad dtype %d", dtype);
  if (vc < 1 || c->nx / 2 < vc || c->ny / 2 < vc || c->nz / 2 < vc)
    return fail(c, BCMG_USAGE, "vc=%d must satisfy 1 <= vc <= size/2 (DataClass.h:53)", vc);
  Field f;
  f.dtype = dtype;
  f.vc = vc;
  const int64_t n0 = c->nx + 2 * vc, n1 = c->ny + 2 * vc, n2 = c->nz + 2 * vc;
  f.brick = n0 * n1 * n2;
  const int64_t align = 256 / (int64_t)dsize(dtype);
  f.bstride = (f.brick + align - 1) / align * align;
  f.bytes = (size_t)f.bstride * c->nb * dsize(dtype);
  if (host) {
    // page-locked, mapped; with unified addressing the host pointer is the
    // device pointer too, which kernels and host code then share
    cudaError_t e = cudaHostAlloc(&f.d, f.bytes ? f.bytes : 1,
                                  cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(c, BCMG_MEMORY, "cudaHostAlloc(%zu): %s", f.bytes, cudaGetErrorString(e));
    }
    void* dp = nullptr;
    if (cudaHostGetDevicePointer(&dp, f.d, 0) != cudaSuccess || dp != f.d) {
      cudaGetLastError();
      cudaFreeHost(f.d);
      return fail(c, BCMG_CUDA_ERROR, "host field: the device does not share the host's addresses");
    }
    f.host = true;
    std::memset(f.d, 0, f.bytes);
  } else {
    int rc = dev_alloc(c, &f.d, f.bytes);
    if (rc) return rc;
    CUDA_TRY(c, cudaMemsetAsync(f.d, 0, f.bytes, c->stream));
  }
  CUDA_TRY(c, cudaEventCreateWithFlags(&f.ev, cudaEventDisableTiming));
  const int h = c->next_field++;
  c->fields[h] = f;
  *out = h;
  return BCMG_SUCCESS;
}

static int work_field(bcmg_ctx c, int dtype, int vc, int slot, int* out) {
  const long key = ((long)dtype * 64 + vc) * 64 + slot;
  auto it = c->work.find(key);
  if (it != c->work.end() && c->fields.count(it->second)) {
    *out = it->second;
    return BCMG_SUCCESS;
  }
  int rc = create_field(c, dtype, vc, out);
  if (rc) return rc;
  c->work[key] = *out;
  return BCMG_SUCCESS;
}

// ---------------------------------------------------------------------------
extern "C" {

BCMG_API int bcmg_ctx_create(bcmg_ctx* out, int device) {
  if (!out) return BCMG_USAGE;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return BCMG_NO_DEVICE;
  }
  if (device < 0 || device >= n) return BCMG_USAGE;
  bcmg_ctx c = new (std::nothrow) bcmg_ctx_s;
  if (!c) return BCMG_MEMORY;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_scalar, 64 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->d_err, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&c->h_scalar, 64 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return BCMG_NO_DEVICE;
  }
  *out = c;
  return BCMG_SUCCESS;
}

BCMG_API void bcmg_ctx_destroy(bcmg_ctx c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->fields) {
    if (kv.second.host) cudaFreeHost(kv.second.d);
    else cudaFree(kv.second.d);
    if (kv.second.ev) cudaEventDestroy(kv.second.ev);
  }
  for (auto& kv : c->ops) {
    cudaFree(kv.second.d_cc);
    cudaFree(kv.second.d_jc32);
    cudaFree(kv.second.d_jc64);
  }
  for (void* q : c->retired) cudaFree(q);
  cudaFree(c->d_tasks);
  cudaFree(c->d_push_ptr);
  cudaFree(c->d_push_tasks);
  cudaFree(c->d_fed);
  cudaFree(c->d_facein);
  cudaFree(c->d_binfo);
  cudaFree(c->d_out_tasks);
  cudaFree(c->d_side[0]);
  cudaFree(c->d_side[1]);
  cudaFree(c->d_bctype);
  cudaFree(c->d_bcval);
  cudaFree(c->d_bczero);
  cudaFree(c->d_bcv2f);
  cudaFree(c->d_bczero2f);
  cudaFree(c->d_partial);
  cudaFree(c->d_scalar);
  cudaFree(c->d_kpart);
  cudaFree(c->d_kseg);
  cudaFreeHost(c->h_kseg);
  cudaFree(c->d_seg_of);
  cudaFree(c->d_seg_first);
  cudaFree(c->d_segflag);
  cudaFree(c->d_segscale);
  cudaFree(c->d_segmaxit);
  cudaFree(c->d_segsum);
  cudaFreeHost(c->h_segsum);
  cudaFree(c->d_err);
  cudaFreeHost(c->h_scalar);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second.exec);
  cudaStreamDestroy(c->stream);
  delete c;
}

BCMG_API const char* bcmg_last_error(bcmg_ctx c) { return c ? c->err.c_str() : "null context"; }

// After a synchronisation: a device-side bounded wait that gave up (its
// kernel recorded the code and returned) fails the call that launched it.
static int take_dev_err(bcmg_ctx c, const char* what) {
  int err = 0;
  CUDA_TRY(c, cudaMemcpy(&err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (!err) return BCMG_SUCCESS;
  CUDA_TRY(c, cudaMemset(c->d_err, 0, sizeof(int)));
  return fail(c, BCMG_CUDA_ERROR, "%s: device-side wait gave up (code 0x%x); results incomplete",
              what, err);
}

BCMG_API int bcmg_sync(bcmg_ctx c, void* st) {
  if (!c) return BCMG_USAGE;
  CUDA_TRY(c, cudaStreamSynchronize(S(c, st)));
  return take_dev_err(c, "bcmg_sync");
}

BCMG_API int bcmg_set_memory_budget(bcmg_ctx c, size_t bytes) {
  if (!c) return BCMG_USAGE;
  c->budget = bytes;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_memory_in_use(bcmg_ctx c, size_t* bytes) {
  if (!c || !bytes) return BCMG_USAGE;
  *bytes = c->in_use;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_profile_begin(bcmg_ctx c) {
  if (!c) return BCMG_USAGE;
  CUDA_TRY(c, cudaDeviceSynchronize());
  c->ev_used = 0;
  c->ev_kind.clear();
  c->profiling = true;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_profile_end(bcmg_ctx c, double* ms_by_kind, int64_t* count_by_kind) {
  if (!c || !ms_by_kind || !count_by_kind) return BCMG_USAGE;
  CUDA_TRY(c, cudaDeviceSynchronize());
  for (int k = 0; k < K_NKINDS; k++) { ms_by_kind[k] = 0.0; count_by_kind[k] = 0; }
  for (size_t p = 0; p < c->ev_kind.size() && 2 * p + 1 < c->ev_used; p++) {
    float ms = 0.f;
    CUDA_TRY(c, cudaEventElapsedTime(&ms, c->ev_pool[2 * p], c->ev_pool[2 * p + 1]));
    ms_by_kind[c->ev_kind[p]] += ms;
    count_by_kind[c->ev_kind[p]] += 1;
  }
  c->profiling = false;
  c->ev_used = 0;
  c->ev_kind.clear();
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_launch_count(bcmg_ctx c, int64_t* n) {
  if (!c || !n) return BCMG_USAGE;
  *n = c->launches;
  return BCMG_SUCCESS;
}

static int check_block_shape(bcmg_ctx c, int nx, int ny, int nz) {
  if (c->registered) return fail(c, BCMG_USAGE, "blocks already registered");
  if (nx < 2 || ny < 2 || nz < 2 || nx % 2 || ny % 2 || nz % 2)
    return fail(c, BCMG_FAILURE, "cell counts must be even and >= 2 (BlockBase.h:76-79)");
  if ((int64_t)nx * ny * nz > (1 << 24)) return fail(c, BCMG_USAGE, "block too large");
  return BCMG_SUCCESS;
}

// Registration once c->ld/id/sf hold the neighbour table of c->nb blocks.
static int finish_register(bcmg_ctx c, int nx, int ny, int nz) {
  const int nb = c->nb;
  c->nx = nx; c->ny = ny; c->nz = nz;
  c->registered = true;
  c->nseg = 1;
  c->seg_first.assign({0, nb});
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaMalloc(&c->d_partial, (size_t)nb * sizeof(double)));
  CUDA_TRY(c, cudaMalloc(&c->d_bczero, (size_t)nb * 6 * sizeof(double)));
  CUDA_TRY(c, cudaMemset(c->d_bczero, 0, (size_t)nb * 6 * sizeof(double)));
  CUDA_TRY(c, cudaMalloc(&c->d_bcval, (size_t)nb * 6 * sizeof(double)));
  CUDA_TRY(c, cudaMemset(c->d_bcval, 0, (size_t)nb * 6 * sizeof(double)));
  CUDA_TRY(c, cudaMalloc(&c->d_bctype, (size_t)nb * 6 * sizeof(int)));
  CUDA_TRY(c, cudaMemset(c->d_bctype, 0, (size_t)nb * 6 * sizeof(int)));
  CUDA_TRY(c, cudaMalloc(&c->d_bcv2f, (size_t)nb * 8 * sizeof(float)));
  CUDA_TRY(c, cudaMemset(c->d_bcv2f, 0, (size_t)nb * 8 * sizeof(float)));
  CUDA_TRY(c, cudaMalloc(&c->d_bczero2f, (size_t)nb * 8 * sizeof(float)));
  CUDA_TRY(c, cudaMemset(c->d_bczero2f, 0, (size_t)nb * 8 * sizeof(float)));
  return build_face_table(c);
}

BCMG_API int bcmg_register_blocks(bcmg_ctx c, int nb, int nx, int ny, int nz, const int* ld,
                                  const int* id, const int* sf) {
  if (!c) return BCMG_USAGE;
  if (int rc = check_block_shape(c, nx, ny, nz)) return rc;
  if (nb <= 0) return fail(c, BCMG_FAILURE, "number of blocks must be > 0 (BlockManager.cpp:38-41)");
  if (!ld || !id || !sf) return fail(c, BCMG_USAGE, "null neighbour table");
  for (int k = 0; k < nb * 6; k++) {
    if (ld[k] < -1 || ld[k] > 1)
      return fail(c, BCMG_FAILURE, "block %d face %d: level difference %d not in -1..1", k / 6,
                  k % 6, ld[k]);
    if (sf[k] < 0 || sf[k] > 3)
      return fail(c, BCMG_FAILURE, "block %d face %d: subface %d", k / 6, k % 6, sf[k]);
    for (int s = 0; s < 4; s++)
      if (id[k * 4 + s] < -1 || id[k * 4 + s] >= nb)
        return fail(c, BCMG_FAILURE, "block %d face %d: neighbour id %d out of range", k / 6,
                    k % 6, id[k * 4 + s]);
  }
  c->nb = nb;
  c->ld.assign(ld, ld + nb * 6);
  c->id.assign(id, id + nb * 24);
  c->sf.assign(sf, sf + nb * 6);
  return finish_register(c, nx, ny, nz);
}

// ---- device-side mesh set-up (mesh_dev.cu) ----
static bool valid_rootgrid(const bcmg_rootgrid* rg) {
  return rg && rg->nx > 0 && rg->ny > 0 && rg->nz > 0 &&
         (long)rg->nx * rg->ny * rg->nz <= 0xfff + 1 && rg->root_length > 0;
}

// Registers the meshes the device set-up made, one after another (block ids
// of mesh i shifted by the blocks before it; first[i] its first block), their
// tables copied to the host for the host-side checks; frees them.
static int adopt_meshes(bcmg_ctx c, std::vector<MeshDev>& ms, int nx, int ny, int nz,
                        int* first) {
  size_t nb = 0;
  for (const MeshDev& m : ms) nb += (size_t)m.nb;
  cudaError_t e = cudaSuccess;
  if (nb == 0 || nb > (size_t)INT32_MAX / 24) {
    for (MeshDev& m : ms) mesh_free(&m, c->stream);
    return fail(c, BCMG_FAILURE, nb ? "too many blocks" : "the mesh has no active block");
  }
  c->peds.resize(nb);
  c->ld.resize(nb * 6);
  c->id.resize(nb * 24);
  c->sf.resize(nb * 6);
  c->outer.resize(nb * 6);
  size_t off = 0;
  for (size_t i = 0; i < ms.size(); i++) {
    MeshDev& m = ms[i];
    const size_t n = (size_t)m.nb;
    if (first) first[i] = (int)off;
    if (e == cudaSuccess && n)
      e = cudaMemcpy(c->peds.data() + off, m.peds, n * sizeof(uint64_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n)
      e = cudaMemcpy(c->ld.data() + off * 6, m.ld, n * 6 * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n)
      e = cudaMemcpy(c->id.data() + off * 24, m.id, n * 24 * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n)
      e = cudaMemcpy(c->sf.data() + off * 6, m.sf, n * 6 * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n)
      e = cudaMemcpy(c->outer.data() + off * 6, m.outer, n * 6 * sizeof(int),
                     cudaMemcpyDeviceToHost);
    if (off)
      for (size_t q = off * 24; q < (off + n) * 24; q++)
        if (c->id[q] >= 0) c->id[q] += (int)off;
    off += n;
    mesh_free(&m, c->stream);
  }
  if (e != cudaSuccess) return fail(c, BCMG_CUDA_ERROR, "mesh set-up: %s", cudaGetErrorString(e));
  c->nb = (int)nb;
  return finish_register(c, nx, ny, nz);
}

static int adopt_mesh(bcmg_ctx c, MeshDev& m, int nx, int ny, int nz) {
  std::vector<MeshDev> ms(1, m);
  m = MeshDev{};
  return adopt_meshes(c, ms, nx, ny, nz, nullptr);
}

static int check_divider(bcmg_ctx c, const bcmg_rootgrid* rg, const bcmg_divider* div) {
  if (!valid_rootgrid(rg) || !div) return fail(c, BCMG_USAGE, "bad root grid or divider");
  if (div->max_level < 0 || div->max_level > 15 || div->min_level < 0 ||
      div->min_level > div->max_level)
    return fail(c, BCMG_USAGE, "divider levels out of 0..15");
  if (div->kind == BCMG_DIV_BALLS && div->npoints > 0 && !div->points)
    return fail(c, BCMG_USAGE, "null points");
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_mesh_build_batch(bcmg_ctx c, int k, const bcmg_rootgrid* rgs,
                                   const bcmg_divider* divs, int nx, int ny, int nz, int* first) {
  if (!c) return BCMG_USAGE;
  if (int rc = check_block_shape(c, nx, ny, nz)) return rc;
  if (k <= 0 || !rgs || !divs) return fail(c, BCMG_USAGE, "no meshes");
  for (int i = 0; i < k; i++)
    if (int rc = check_divider(c, &rgs[i], &divs[i])) return rc;
  CUDA_TRY(c, cudaSetDevice(c->device));
  std::vector<MeshDev> ms(k);
  for (int i = 0; i < k; i++) {
    const char* why = "";
    const int rc = mesh_from_divider(rgs[i], divs[i], &ms[i], c->stream, &why);
    if (rc != BCMG_SUCCESS) {
      for (MeshDev& m : ms) mesh_free(&m, c->stream);
      return fail(c, rc, "mesh set-up of mesh %d: %s", i, why);
    }
  }
  return adopt_meshes(c, ms, nx, ny, nz, first);
}

BCMG_API int bcmg_mesh_build(bcmg_ctx c, const bcmg_rootgrid* rg, const bcmg_divider* div, int nx,
                             int ny, int nz) {
  if (!c) return BCMG_USAGE;
  if (int rc = check_block_shape(c, nx, ny, nz)) return rc;
  if (int rc = check_divider(c, rg, div)) return rc;
  CUDA_TRY(c, cudaSetDevice(c->device));
  MeshDev m;
  const char* why = "";
  const int rc = mesh_from_divider(*rg, *div, &m, c->stream, &why);
  if (rc != BCMG_SUCCESS) return fail(c, rc, "mesh set-up: %s", why);
  return adopt_mesh(c, m, nx, ny, nz);
}

BCMG_API int bcmg_mesh_register_pedigrees(bcmg_ctx c, const bcmg_rootgrid* rg,
                                          const uint64_t* peds, int n, int balance, int nx,
                                          int ny, int nz) {
  if (!c) return BCMG_USAGE;
  if (int rc = check_block_shape(c, nx, ny, nz)) return rc;
  if (!valid_rootgrid(rg) || n <= 0 || !peds) return fail(c, BCMG_USAGE, "bad root grid or leaf list");
  CUDA_TRY(c, cudaSetDevice(c->device));
  MeshDev m;
  const char* why = "";
  const int rc = mesh_from_pedigrees(*rg, peds, n, balance != 0, &m, c->stream, &why);
  if (rc != BCMG_SUCCESS) return fail(c, rc, "mesh set-up: %s", why);
  return adopt_mesh(c, m, nx, ny, nz);
}

// ---- ghost exchange with other processes (Scalar3DUpdater.h:377-515,
// 711-901): the entries as face-table entries, their offsets in the buffer ----
static int xch_entries(bcmg_ctx c, const Field& f, const bcmg_xch_entry* e, int n, bool pack,
                       std::vector<VcTask>* tasks, std::vector<int64_t>* off, size_t* bytes) {
  if (n < 0 || (n > 0 && !e)) return fail(c, BCMG_USAGE, "exchange: bad entry list");
  tasks->resize(n);
  off->resize(n);
  int64_t at = 0;
  const int64_t vc = f.vc;
  for (int q = 0; q < n; q++) {
    const bcmg_xch_entry& x = e[q];
    if (x.block < 0 || x.block >= c->nb || x.face < 0 || x.face > 5 || x.subface < 0 ||
        x.subface > 3 || x.kind < BCMG_XCH_COPY || x.kind > BCMG_XCH_C2F)
      return fail(c, BCMG_USAGE, "exchange entry %d: block %d face %d subface %d kind %d", q,
                  x.block, x.face, x.subface, x.kind);
    VcTask t{};
    t.face = (uint8_t)x.face;
    t.subface = (uint8_t)x.subface;
    t.kind = x.kind == BCMG_XCH_COPY ? VC_COPY : x.kind == BCMG_XCH_F2C ? VC_F2C : VC_C2F;
    t.dst = pack ? 0 : x.block;
    t.src = pack ? x.block : -1;
    t.slot = -1;
    (*tasks)[q] = t;
    (*off)[q] = at;
    const int ax = x.face / 2;
    const int64_t n0 = ax == 0 ? c->ny : c->nx, n1 = ax == 2 ? c->ny : c->nz;
    at += x.kind == BCMG_XCH_F2C ? vc * (n0 / 2) * (n1 / 2) : vc * n0 * n1;
  }
  *bytes = (size_t)at * dsize(f.dtype);
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_xch_bytes(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n,
                            size_t* bytes) {
  if (!c || !bytes) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "bad field id");
  std::vector<VcTask> tasks;
  std::vector<int64_t> off;
  return xch_entries(c, *f, e, n, true, &tasks, &off, bytes);
}

static int xch_run(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n, void* buf, bool pack,
                   void* stream) {
  if (!c || (n > 0 && !buf)) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "bad field id");
  std::vector<VcTask> tasks;
  std::vector<int64_t> off;
  size_t bytes = 0;
  if (int rc = xch_entries(c, *f, e, n, pack, &tasks, &off, &bytes)) return rc;
  if (n == 0) return BCMG_SUCCESS;
  cudaStream_t st = S(c, stream);
  VcTask* d_t = nullptr;
  int64_t* d_o = nullptr;
  CUDA_TRY(c, cudaMallocAsync(reinterpret_cast<void**>(&d_t), tasks.size() * sizeof(VcTask), st));
  CUDA_TRY(c, cudaMallocAsync(reinterpret_cast<void**>(&d_o), off.size() * sizeof(int64_t), st));
  CUDA_TRY(c, cudaMemcpyAsync(d_t, tasks.data(), tasks.size() * sizeof(VcTask),
                              cudaMemcpyHostToDevice, st));
  CUDA_TRY(c, cudaMemcpyAsync(d_o, off.data(), off.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice, st));
  const Geom g = geom_of(c, *f);
  if (f->dtype == BCMG_F64)
    LAUNCH(c, K_VC, st, launch_xch<double>((double*)f->d, g, d_t, d_o, n, (double*)buf, pack, st));
  else
    LAUNCH(c, K_VC, st, launch_xch<float>((float*)f->d, g, d_t, d_o, n, (float*)buf, pack, st));
  cudaFreeAsync(d_t, st);
  cudaFreeAsync(d_o, st);
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_xch_pack(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n, void* buf,
                           void* stream) {
  return xch_run(c, field, e, n, buf, true, stream);
}

BCMG_API int bcmg_xch_unpack(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n,
                             const void* buf, void* stream) {
  return xch_run(c, field, e, n, const_cast<void*>(buf), false, stream);
}

BCMG_API int bcmg_num_blocks(bcmg_ctx c, int* nb) {
  if (!c || !nb) return BCMG_USAGE;
  *nb = c->registered ? c->nb : 0;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_mesh_pedigrees(bcmg_ctx c, uint64_t* peds) {
  if (!c || !peds) return BCMG_USAGE;
  if (c->peds.empty()) return fail(c, BCMG_USAGE, "no mesh registered by the device set-up");
  std::memcpy(peds, c->peds.data(), c->peds.size() * sizeof(uint64_t));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_mesh_neighbors(bcmg_ctx c, int* ld, int* id, int* sf, int* outer) {
  if (!c || !ld || !id || !sf) return BCMG_USAGE;
  if (!c->registered) return fail(c, BCMG_USAGE, "no blocks registered");
  std::memcpy(ld, c->ld.data(), c->ld.size() * sizeof(int));
  std::memcpy(id, c->id.data(), c->id.size() * sizeof(int));
  std::memcpy(sf, c->sf.data(), c->sf.size() * sizeof(int));
  if (outer) {
    if (c->outer.empty()) return fail(c, BCMG_USAGE, "outer faces: no mesh registered by the device set-up");
    std::memcpy(outer, c->outer.data(), c->outer.size() * sizeof(int));
  }
  return BCMG_SUCCESS;
}

// Buffers of the per-segment kernel arguments for `nseg` segments.
static int seg_buffers(bcmg_ctx c, int nseg) {
  if (c->segbuf_cap >= nseg) return BCMG_SUCCESS;
  cudaFree(c->d_segflag);
  cudaFree(c->d_segscale);
  cudaFree(c->d_segmaxit);
  cudaFree(c->d_segeps2);
  cudaFree(c->d_segsum);
  cudaFreeHost(c->h_segsum);
  c->d_segeps2 = nullptr;
  c->d_segflag = nullptr;
  c->d_segscale = nullptr;
  c->d_segmaxit = nullptr;
  c->d_segsum = nullptr;
  c->h_segsum = nullptr;
  c->segbuf_cap = 0;
  CUDA_TRY(c, cudaMalloc(&c->d_segflag, (size_t)nseg));
  CUDA_TRY(c, cudaMalloc(&c->d_segscale, (size_t)nseg * sizeof(double)));
  CUDA_TRY(c, cudaMalloc(&c->d_segmaxit, (size_t)nseg * sizeof(int)));
  CUDA_TRY(c, cudaMalloc(&c->d_segeps2, (size_t)nseg * sizeof(double)));
  CUDA_TRY(c, cudaMalloc(&c->d_segsum, (size_t)2 * nseg * sizeof(double)));
  CUDA_TRY(c, cudaMallocHost(&c->h_segsum, (size_t)2 * nseg * sizeof(double)));
  c->segbuf_cap = nseg;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_set_segments(bcmg_ctx c, int nseg, const int* seg_first) {
  if (!c) return BCMG_USAGE;
  if (!c->registered) return fail(c, BCMG_USAGE, "no blocks registered");
  if (nseg < 1 || !seg_first) return fail(c, BCMG_USAGE, "need at least one segment");
  if (seg_first[0] != 0 || seg_first[nseg] != c->nb)
    return fail(c, BCMG_USAGE, "segments must cover blocks [0, %d)", c->nb);
  for (int q = 0; q < nseg; q++)
    if (seg_first[q + 1] <= seg_first[q])
      return fail(c, BCMG_USAGE, "segment %d is empty or out of order", q);
  // no face may join blocks of two segments: they are independent systems
  for (int b = 0, q = 0; b < c->nb; b++) {
    while (b >= seg_first[q + 1]) q++;
    for (int k = 0; k < 24; k++) {
      const int n = c->id[(size_t)b * 24 + k];
      if (n >= 0 && (n < seg_first[q] || n >= seg_first[q + 1]))
        return fail(c, BCMG_USAGE, "block %d (segment %d) has neighbour %d in another segment",
                    b, q, n);
    }
  }
  std::vector<int> of(c->nb);
  for (int q = 0; q < nseg; q++)
    for (int b = seg_first[q]; b < seg_first[q + 1]; b++) of[b] = q;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  cudaFree(c->d_seg_of);
  cudaFree(c->d_seg_first);
  c->d_seg_of = nullptr;
  c->d_seg_first = nullptr;
  c->nseg = 1;
  c->seg_first.assign({0, c->nb});
  if (nseg > 1) {
    CUDA_TRY(c, cudaMalloc(&c->d_seg_of, (size_t)c->nb * sizeof(int)));
    CUDA_TRY(c, cudaMalloc(&c->d_seg_first, (size_t)(nseg + 1) * sizeof(int)));
    CUDA_TRY(c, cudaMemcpy(c->d_seg_of, of.data(), (size_t)c->nb * sizeof(int),
                           cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_seg_first, seg_first, (size_t)(nseg + 1) * sizeof(int),
                           cudaMemcpyHostToDevice));
    c->nseg = nseg;
    c->seg_first.assign(seg_first, seg_first + nseg + 1);
  }
  return seg_buffers(c, c->nseg);
}

BCMG_API int bcmg_set_boundary(bcmg_ctx c, const int* bc_type, const double* bc_value, int form) {
  if (!c) return BCMG_USAGE;
  if (!c->registered) return fail(c, BCMG_USAGE, "no blocks registered");
  if (!bc_type || !bc_value) return fail(c, BCMG_USAGE, "null boundary table");
  if (form != BCMG_DIRICHLET_SOR && form != BCMG_DIRICHLET_BCX)
    return fail(c, BCMG_USAGE, "bad Dirichlet form %d", form);
  for (int k = 0; k < c->nb * 6; k++)
    if (bc_type[k] < 0 || bc_type[k] > 3)
      return fail(c, BCMG_USAGE, "bad boundary type %d", bc_type[k]);
  c->bctype.assign(bc_type, bc_type + c->nb * 6);
  c->bcval.assign(bc_value, bc_value + c->nb * 6);
  c->bcform = form;
  CUDA_TRY(c, cudaMemcpy(c->d_bctype, bc_type, (size_t)c->nb * 6 * sizeof(int),
                         cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->d_bcval, bc_value, (size_t)c->nb * 6 * sizeof(double),
                         cudaMemcpyHostToDevice));
  {
    std::vector<float> v2f((size_t)c->nb * 8, 0.0f);
    for (size_t b = 0; b < (size_t)c->nb; b++)
      for (int f = 0; f < 6; f++) {
        double v = bc_value[b * 6 + f];
        if (form == BCMG_DIRICHLET_BCX) v = (double)(float)v;
        const double v2 = 2.0 * v;
        const float w = (float)v2;
        v2f[b * 8 + f] = ((double)w == v2) ? w : std::numeric_limits<float>::quiet_NaN();
      }
    CUDA_TRY(c, cudaMemcpy(c->d_bcv2f, v2f.data(), v2f.size() * sizeof(float),
                           cudaMemcpyHostToDevice));
  }
  return build_face_table(c);
}

BCMG_API int bcmg_field_create(bcmg_ctx c, int dtype, int vc, int* field) {
  if (!c || !field) return BCMG_USAGE;
  return create_field(c, dtype, vc, field);
}

BCMG_API int bcmg_field_create_host(bcmg_ctx c, int dtype, int vc, int* field) {
  if (!c || !field) return BCMG_USAGE;
  return create_field(c, dtype, vc, field, true);
}

// Fields in host memory serve host code that sweeps its own bricks and
// hands the ghost update to the device (the C++ drop-in headers).  The sweep
// kernels stage bricks with bulk asynchronous copies, which this library
// issues on device memory only: those entry points refuse host fields.
static int refuse_host(bcmg_ctx c, std::initializer_list<int> ids, const char* what) {
  for (int id : ids) {
    const Field* f = get_field(c, id);
    if (f && f->host)
      return fail(c, BCMG_USAGE,
                  "%s: field %d lives in host memory (bcmg_field_create_host); sweeps and "
                  "solvers need device fields", what, id);
  }
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_destroy(bcmg_ctx c, int field) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  cudaStreamSynchronize(c->stream);
  clear_graphs(c);  // captured runs may refer to this memory
  if (f->host) cudaFreeHost(f->d);
  else dev_free(c, f->d, f->bytes);
  if (f->ev) cudaEventDestroy(f->ev);
  c->fields.erase(field);
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_layout(bcmg_ctx c, int field, void** dptr, int64_t* bstride,
                               int64_t* brick) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  if (dptr) *dptr = f->d;
  if (bstride) *bstride = f->bstride;
  if (brick) *brick = f->brick;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_upload(bcmg_ctx c, int field, const void* host, void* st) {
  if (!c || !host) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  const size_t es = dsize(f->dtype);
  const cudaMemcpyKind kind = f->host ? cudaMemcpyDefault : cudaMemcpyHostToDevice;
  if (f->bstride == f->brick)  // unpadded bricks: one linear copy
    CUDA_TRY(c, cudaMemcpyAsync(f->d, host, f->bytes, kind, S(c, st)));
  else
    CUDA_TRY(c, cudaMemcpy2DAsync(f->d, f->bstride * es, host, f->brick * es, f->brick * es,
                                  c->nb, kind, S(c, st)));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_download(bcmg_ctx c, int field, void* host, void* st) {
  if (!c || !host) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  const size_t es = dsize(f->dtype);
  const cudaMemcpyKind kind = f->host ? cudaMemcpyDefault : cudaMemcpyDeviceToHost;
  if (f->bstride == f->brick)  // unpadded bricks: one linear copy
    CUDA_TRY(c, cudaMemcpyAsync(host, f->d, f->bytes, kind, S(c, st)));
  else
    CUDA_TRY(c, cudaMemcpy2DAsync(host, f->brick * es, f->d, f->bstride * es, f->brick * es,
                                  c->nb, kind, S(c, st)));
  CUDA_TRY(c, cudaStreamSynchronize(S(c, st)));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_fill(bcmg_ctx c, int field, double v, void* st) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  const int64_t n = f->bstride * c->nb;
  if (f->dtype == BCMG_F64) LAUNCH(c, K_FILL, S(c, st), launch_fill<double>((double*)f->d, n, v, S(c, st)));
  else LAUNCH(c, K_FILL, S(c, st), launch_fill<float>((float*)f->d, n, (float)v, S(c, st)));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_fill_random(bcmg_ctx c, int field, int first_block, int nblocks,
                                    uint64_t seed, double lo, double hi, void* st) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  if (first_block < 0 || nblocks < 0 || first_block + nblocks > c->nb)
    return fail(c, BCMG_USAGE, "block range [%d, %d) outside [0, %d)", first_block,
                first_block + nblocks, c->nb);
  Geom g = geom_of(c, *f);
  if (f->dtype == BCMG_F64)
    LAUNCH(c, K_FILL, S(c, st), launch_fill_random<double>((double*)f->d, g, first_block, nblocks,
                                                           seed, lo, hi, S(c, st)));
  else
    LAUNCH(c, K_FILL, S(c, st), launch_fill_random<float>((float*)f->d, g, first_block, nblocks,
                                                          seed, lo, hi, S(c, st)));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_copy(bcmg_ctx c, int dst, int src, void* st) {
  if (!c) return BCMG_USAGE;
  Field *d = get_field(c, dst), *s = get_field(c, src);
  if (!d || !s) return fail(c, BCMG_USAGE, "unknown field");
  if (d->dtype != s->dtype || d->vc != s->vc) return fail(c, BCMG_USAGE, "field shapes differ");
  CUDA_TRY(c, cudaMemcpyAsync(d->d, s->d, d->bytes,
                              d->host || s->host ? cudaMemcpyDefault : cudaMemcpyDeviceToDevice,
                              S(c, st)));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_field_swap(bcmg_ctx c, int a, int b) {
  if (!c) return BCMG_USAGE;
  Field *fa = get_field(c, a), *fb = get_field(c, b);
  if (!fa || !fb) return fail(c, BCMG_USAGE, "unknown field");
  if (fa->dtype != fb->dtype || fa->vc != fb->vc) return fail(c, BCMG_USAGE, "field shapes differ");
  if (fa->host != fb->host) return fail(c, BCMG_USAGE, "cannot swap a host field with a device field");
  std::swap(fa->d, fb->d);
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_prepare_vc(bcmg_ctx c, int field, int tag, int method) {
  (void)tag;  // MPI message tag of the reference; no messages on one rank
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  if (method < BCMG_VC_AT_ONCE || method > BCMG_VC_SEPARATE_XYZ_LEVELDIFF)
    return fail(c, BCMG_USAGE, "bad VC method %d", method);
  f->vc_method = method;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_vc_begin(bcmg_ctx c, int field, int axis_mask, int ld_mask, void* st) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  if (f->vc_method < 0)
    return fail(c, BCMG_USAGE, "prepareForVCUpdate was not called for field %d", field);
  int rc = gather(c, *f, select_ranges(c, axis_mask & 7, ld_mask & 7, true, false), false, S(c, st));
  if (rc) return rc;
  CUDA_TRY(c, cudaEventRecord(f->ev, S(c, st)));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_vc_end(bcmg_ctx c, int field) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  CUDA_TRY(c, cudaEventSynchronize(f->ev));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_bc_apply(bcmg_ctx c, int field, void* st) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  return gather(c, *f, select_ranges(c, 7, 7, false, true), false, S(c, st));
}

BCMG_API int bcmg_impose_bc(bcmg_ctx c, int field, void* st) {
  if (!c) return BCMG_USAGE;
  Field* f = get_field(c, field);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", field);
  return impose(c, *f, false, S(c, st));
}

// Fewest outer iterations for which a fused pull-form SOR run packs its source.
constexpr int kPackMinIters = 8;

static long sor_key(int dtype, int n, int vc, int form) {
  return ((long)(dtype * 64 + n) * 8 + vc) * 4 + form;
}

// Kernel shape for a fused SOR sweep: forced, tuned, or the default -- the
// pull form one CTA per block (7) where it applies, else the staged-source
// tile (1).  Push-only
// contexts (bcmg_set_ghost_form) never get the pull form.
static int sor_variant(bcmg_ctx c, const Field& f, int form) {
  const bool cubic = c->nx == c->ny && c->ny == c->nz;
  const bool pull_ok = c->ghost_form != BCMG_GHOST_PUSH && cubic && sor_pull_ok((int)dsize(f.dtype), c->nx, f.vc, form);
  int v = c->sor_fixed;
  if (!v) {
    auto it = c->sor_tuned.find(sor_key(f.dtype, c->nx, f.vc, form));
    v = it == c->sor_tuned.end() ? (pull_ok ? SV_PULL_TILE : SV_TILE_SS_256) : it->second;
  }
  if ((v == SV_PULL || v == SV_PULL_TILE) && !pull_ok) v = SV_TILE_SS_256;
  return v;
}

// ---------------------------------------------------------------------------
BCMG_API int bcmg_sor_run(bcmg_ctx c, int fid, int sid, const double* coef, double omega,
                          int form, int n_inner, int n_outer, void* st) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {fid, sid}, "bcmg_sor_run")) return rc_host;
  Field* f = get_field(c, fid);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", fid);
  Field* s = nullptr;
  if (form == 2) {
    s = get_field(c, sid);
    if (!s || s->dtype != f->dtype || s->vc != f->vc)
      return fail(c, BCMG_USAGE, "form 2 needs a source field shaped like f");
  } else if (form != 1) {
    return fail(c, BCMG_USAGE, "bad SOR form %d", form);
  }
  if (!coef || n_inner < 0 || n_outer < 0) return fail(c, BCMG_USAGE, "bad SOR arguments");
  if (c->has_neumann)
    return fail(c, BCMG_FAILURE,
                "Neumann boundary condition is not implemented in the SOR schemes "
                "(sor1/Solver.cpp:214-221)");
  cudaStream_t stream = S(c, st);
  // Device copy of the coefficients: nb*4 doubles followed by the same values
  // rounded to float (the FP32 sweep's operands).
  double* d_coef = nullptr;
  const size_t nc = (size_t)c->nb * 4;
  const size_t cb = nc * sizeof(double) + nc * sizeof(float);
  std::vector<unsigned char> hc(cb);
  std::memcpy(hc.data(), coef, nc * sizeof(double));
  for (size_t k = 0; k < nc; k++) {
    const float v = (float)coef[k];
    std::memcpy(hc.data() + nc * sizeof(double) + k * sizeof(float), &v, sizeof(float));
  }
  CUDA_TRY(c, cudaMallocAsync((void**)&d_coef, cb, stream));
  CUDA_TRY(c, cudaMemcpyAsync(d_coef, hc.data(), cb, cudaMemcpyHostToDevice, stream));
  CUDA_TRY(c, cudaStreamSynchronize(stream));  // hc is pageable and goes out of scope
  Geom g = geom_of(c, *f);
  BlockBc bbc{c->bctype.empty() ? nullptr : c->d_bctype, c->d_bcval,
              c->bcform == BCMG_DIRICHLET_BCX ? 1 : 0, c->d_bcv2f};
  const size_t es = dsize(f->dtype);
  const int variant = sor_variant(c, *f, form);
  int rc0;
  const bool pulled = variant == SV_PULL || variant == SV_PULL_TILE;
  if (pulled && (rc0 = ensure_side(c, es))) {
    cudaFreeAsync(d_coef, stream);
    return rc0;
  }
  PushTable pt = push_table(c, 0);
  const size_t smem = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2) * es;
  // Fused ping-pong path: one launch per outer iteration writes the next
  // iterate with every ghost updated.  It needs the block's Dirichlet ghosts
  // to be the only writers of their cells (no Dirichlet face with a
  // neighbour), at least one inner pass, and a brick that fits shared memory.
  const bool fused = n_inner >= 1 && !c->bc_conflict && smem <= kSorMaxSmem && !c->no_fusion;
  int rc = BCMG_SUCCESS;
  if (fused && n_outer > 0) {
    int wid, pid = -1;
    if ((rc = work_field(c, f->dtype, f->vc, 30, &wid))) { cudaFreeAsync(d_coef, stream); return rc; }
    // Runs of the pull-form kernels with a source term and enough iterations
    // read the source packed N^3 per block in sweep order (no padding, one
    // bulk copy per block): packed once here, it saves the padding's bytes
    // on every iteration.
    bool pack = pulled && form == 2 && n_outer >= kPackMinIters;
    if (pack && (rc = work_field(c, f->dtype, f->vc, 34, &pid))) {
      if (rc != BCMG_MEMORY) {
        cudaFreeAsync(d_coef, stream);
        return rc;
      }
      pack = false;  // no room for the packed copy: read the source as it is
      rc = BCMG_SUCCESS;
    }
    f = get_field(c, fid);
    s = form == 2 ? get_field(c, sid) : nullptr;
    Field* w = get_field(c, wid);
    const void* sd = s ? s->d : nullptr;
    if (pack) {
      Field* pf = get_field(c, pid);
      prof_mark(c, K_FILL, stream, true);
      cudaError_t e = f->dtype == BCMG_F64
                          ? launch_pack_source<double>((double*)pf->d, (const double*)s->d, g, stream)
                          : launch_pack_source<float>((float*)pf->d, (const float*)s->d, g, stream);
      prof_mark(c, K_FILL, stream, false);
      c->launches++;
      if (e != cudaSuccess) {
        cudaFreeAsync(d_coef, stream);
        return fail(c, BCMG_CUDA_ERROR, "source packing: %s", cudaGetErrorString(e));
      }
      sd = pf->d;
    }
    // Cells no kernel writes (edges, corners, ghosts without a source) must
    // agree between the two buffers: start from a copy.
    CUDA_TRY(c, cudaMemcpyAsync(w->d, f->d, f->bytes, cudaMemcpyDeviceToDevice, stream));
    Field* A = f;
    Field* B = w;
    for (int it = 0; it < n_outer; it++) {
      cudaError_t e;
      const int pull_now = it > 0 ? 1 : 0;
      pt = push_table(c, it);
      prof_mark(c, K_SOR, stream, true);
      if (f->dtype == BCMG_F64)
        e = launch_sor<double>((const double*)A->d, (double*)B->d, (const double*)sd, g, d_coef,
                               omega, form, n_inner, bbc, pt, true, c->d_err, variant, pull_now,
                               stream, pack);
      else
        e = launch_sor<float>((const float*)A->d, (float*)B->d, (const float*)sd, g, d_coef,
                              omega, form, n_inner, bbc, pt, true, c->d_err, variant, pull_now,
                              stream, pack);
      prof_mark(c, K_SOR, stream, false);
      c->launches++;
      if (e != cudaSuccess) {
        rc = fail(c, BCMG_CUDA_ERROR, "SOR launch: %s", cudaGetErrorString(e));
        break;
      }
      std::swap(A, B);
    }
    // the pull form leaves the ghosts of fed faces to the reader: update them
    if (rc == BCMG_SUCCESS && pulled) rc = impose(c, *A, false, stream);
    if (rc == BCMG_SUCCESS && A != f)
      CUDA_TRY(c, cudaMemcpyAsync(f->d, A->d, f->bytes, cudaMemcpyDeviceToDevice, stream));
    cudaFreeAsync(d_coef, stream);
    return rc;
  }
  // In-place path: SOR pass, then the gather.  The SOR kernel leaves the
  // block's Dirichlet ghosts final, so after it only the VC update remains
  // (unless a Dirichlet face also has a neighbour).
  const VcRanges after = select_ranges(c, 7, 7, true, n_inner == 0 || c->bc_conflict);
  for (int it = 0; it < n_outer && rc == BCMG_SUCCESS; it++) {
    cudaError_t e;
    prof_mark(c, K_SOR, stream, true);
    if (f->dtype == BCMG_F64)
      e = launch_sor<double>((const double*)f->d, (double*)f->d, s ? (const double*)s->d : nullptr,
                             g, d_coef, omega, form, n_inner, bbc, pt, false, c->d_err, 0, 0, stream);
    else
      e = launch_sor<float>((const float*)f->d, (float*)f->d, s ? (const float*)s->d : nullptr, g,
                            d_coef, omega, form, n_inner, bbc, pt, false, c->d_err, 0, 0, stream);
    prof_mark(c, K_SOR, stream, false);
    c->launches++;
    if (e != cudaSuccess) {
      rc = fail(c, BCMG_CUDA_ERROR, "SOR launch: %s", cudaGetErrorString(e));
      break;
    }
    rc = gather(c, *f, after, false, stream);
  }
  cudaFreeAsync(d_coef, stream);
  return rc;
}

BCMG_API int bcmg_set_sor_variant(bcmg_ctx c, int variant) {
  if (!c) return BCMG_USAGE;
  if (variant < 0 || variant >= SV_COUNT) return fail(c, BCMG_USAGE, "bad SOR variant %d", variant);
  c->sor_fixed = variant;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_autotune_sor(bcmg_ctx c, int fid, int sid, const double* coef, double omega,
                               int form, int iters, int* best, double* best_us) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {fid, sid}, "bcmg_autotune_sor")) return rc_host;
  Field* f = get_field(c, fid);
  if (!f) return fail(c, BCMG_USAGE, "unknown field %d", fid);
  if (iters < 1) iters = 1;
  int tid;
  int rc = work_field(c, f->dtype, f->vc, 31, &tid);
  if (rc) return rc;
  f = get_field(c, fid);
  Field* t = get_field(c, tid);
  cudaEvent_t e0, e1;
  CUDA_TRY(c, cudaEventCreate(&e0));
  CUDA_TRY(c, cudaEventCreate(&e1));
  const int saved = c->sor_fixed;
  int bv = 1;
  double bt = 1e300;
  for (int v = 1; v < SV_COUNT; v++) {
    if ((v == SV_PULL || v == SV_PULL_TILE) && (c->ghost_form == BCMG_GHOST_PUSH || !sor_pull_ok((int)dsize(f->dtype), c->nx, f->vc, form) ||
                         c->nx != c->ny || c->ny != c->nz))
      continue;
    CUDA_TRY(c, cudaMemcpyAsync(t->d, f->d, f->bytes, cudaMemcpyDeviceToDevice, c->stream));
    c->sor_fixed = v;
    rc = bcmg_sor_run(c, tid, sid, coef, omega, form, 1, 1, c->stream);  // warm-up
    if (rc == BCMG_SUCCESS) {
      cudaEventRecord(e0, c->stream);
      rc = bcmg_sor_run(c, tid, sid, coef, omega, form, 1, iters, c->stream);
      cudaEventRecord(e1, c->stream);
    }
    if (rc != BCMG_SUCCESS) break;
    CUDA_TRY(c, cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < bt) { bt = ms; bv = v; }
  }
  c->sor_fixed = saved;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != BCMG_SUCCESS) return rc;
  c->sor_tuned[sor_key(f->dtype, c->nx, f->vc, form)] = bv;
  if (best) *best = bv;
  if (best_us) *best_us = bt * 1e3 / iters;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_set_fusion(bcmg_ctx c, int enable) {
  if (!c) return BCMG_USAGE;
  c->no_fusion = !enable;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_set_ghost_form(bcmg_ctx c, int form) {
  if (!c) return BCMG_USAGE;
  if (form != BCMG_GHOST_PULL && form != BCMG_GHOST_PUSH && form != BCMG_GHOST_AUTO)
    return fail(c, BCMG_USAGE, "bad ghost form %d", form);
  c->ghost_form = form;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_set_jacobi_shape(bcmg_ctx c, int shape) {
  if (!c) return BCMG_USAGE;
  if (shape != 0 && shape != kJacobiTile && shape != kJacobiPipe)
    return fail(c, BCMG_USAGE, "bad Jacobi shape %d", shape);
  c->jacobi_shape = shape;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_op_create_const(bcmg_ctx c, const double* cc, int* op) {
  if (!c || !cc || !op) return BCMG_USAGE;
  if (!c->registered) return fail(c, BCMG_USAGE, "no blocks registered");
  OpRec r;
  const size_t nb = (size_t)c->nb;
  std::vector<float> j32(nb * 8);
  std::vector<double> j64(nb * 8);
  for (size_t b = 0; b < nb; b++) {
    for (int k = 0; k < 7; k++) {
      j32[b * 8 + k] = (float)cc[b * 7 + k];
      j64[b * 8 + k] = cc[b * 7 + k];
    }
    // RN(1/Ap) for the kernels' two-FMA correctly rounded division, only for
    // divisors whose reciprocal keeps every quotient step away from
    // overflow and underflow (0 selects the division instruction sequence)
    const float a32 = std::fabs(j32[b * 8]);
    const double a64 = std::fabs(j64[b * 8]);
    j32[b * 8 + 7] = (a32 >= 0x1p-60f && a32 <= 0x1p+60f) ? 1.0f / j32[b * 8] : 0.0f;
    j64[b * 8 + 7] = (a64 >= 0x1p-60 && a64 <= 0x1p+60) ? 1.0 / j64[b * 8] : 0.0;
  }
  CUDA_TRY(c, cudaMalloc(&r.d_cc, nb * 7 * sizeof(double)));
  CUDA_TRY(c, cudaMalloc(&r.d_jc32, nb * 8 * sizeof(float)));
  CUDA_TRY(c, cudaMalloc(&r.d_jc64, nb * 8 * sizeof(double)));
  CUDA_TRY(c, cudaMemcpy(r.d_cc, cc, nb * 7 * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(r.d_jc32, j32.data(), nb * 8 * sizeof(float), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(r.d_jc64, j64.data(), nb * 8 * sizeof(double), cudaMemcpyHostToDevice));
  *op = c->next_op++;
  c->ops[*op] = r;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_op_create_fields(bcmg_ctx c, const int* f7, int* op) {
  if (!c || !f7 || !op) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {f7[0], f7[1], f7[2], f7[3], f7[4], f7[5], f7[6]},
                                "bcmg_op_create_fields"))
    return rc_host;
  Field* f0 = get_field(c, f7[0]);
  if (!f0) return fail(c, BCMG_USAGE, "unknown coefficient field");
  for (int k = 0; k < 7; k++) {
    Field* f = get_field(c, f7[k]);
    if (!f || f->dtype != f0->dtype || f->vc != f0->vc)
      return fail(c, BCMG_USAGE, "coefficient fields must share dtype and vc");
  }
  OpRec r;
  for (int k = 0; k < 7; k++) r.fields[k] = f7[k];
  *op = c->next_op++;
  c->ops[*op] = r;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_op_destroy(bcmg_ctx c, int op) {
  if (!c) return BCMG_USAGE;
  auto it = c->ops.find(op);
  if (it == c->ops.end()) return fail(c, BCMG_USAGE, "unknown operator %d", op);
  cudaFree(it->second.d_cc);
  cudaFree(it->second.d_jc32);
  cudaFree(it->second.d_jc64);
  c->ops.erase(it);
  return BCMG_SUCCESS;
}

// LocalScalar3D::ImposeBoundaryCondition(Ap..At, b) (SolverTest
// LocalScalar3D.h:260-285): folds the outer Dirichlet and Neumann faces of the
// boundary table into a coefficient-brick operator and the right-hand side.
static bool same_shape(const Field* a, const Field* b);

BCMG_API int bcmg_op_fold_boundary(bcmg_ctx c, int op, int b, void* st) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {b}, "bcmg_op_fold_boundary")) return rc_host;
  auto it = c->ops.find(op);
  if (it == c->ops.end()) return fail(c, BCMG_USAGE, "unknown operator %d", op);
  if (it->second.fields[0] < 0)
    return fail(c, BCMG_USAGE, "folding needs an operator of coefficient fields");
  Field* fb = get_field(c, b);
  Field* f0 = get_field(c, it->second.fields[0]);
  if (!fb || !f0 || !same_shape(fb, f0))
    return fail(c, BCMG_USAGE, "right-hand side must match the coefficient fields");
  for (int k = 0; k < 7; k++) {
    Field* f = get_field(c, it->second.fields[k]);
    if (!f) return fail(c, BCMG_USAGE, "coefficient field %d was destroyed", it->second.fields[k]);
    if (f == fb) return fail(c, BCMG_USAGE, "right-hand side is a coefficient field");
  }
  if (c->bctype.empty()) return BCMG_SUCCESS;
  // outer faces only (BlockScalar3D.h:95-105: faces with a neighbour are INNER)
  std::vector<int> code((size_t)c->nb * 6, 0);
  bool any = false;
  for (size_t k = 0; k < code.size(); k++) {
    const int t = c->bctype[k];
    if (t != BCMG_BC_DIRICHLET && t != BCMG_BC_NEUMANN) continue;
    if (c->id[k * 4] >= 0 || c->id[k * 4 + 1] >= 0 || c->id[k * 4 + 2] >= 0 ||
        c->id[k * 4 + 3] >= 0)
      continue;
    code[k] = t == BCMG_BC_DIRICHLET ? 1 : 2;
    any = true;
  }
  if (!any) return BCMG_SUCCESS;
  cudaStream_t stream = S(c, st);
  int* d_code = nullptr;
  CUDA_TRY(c, cudaMallocAsync((void**)&d_code, code.size() * sizeof(int), stream));
  CUDA_TRY(c, cudaMemcpyAsync(d_code, code.data(), code.size() * sizeof(int),
                              cudaMemcpyHostToDevice, stream));
  Geom g = geom_of(c, *fb);
  int rc = BCMG_SUCCESS;
  cudaError_t e;
  if (fb->dtype == BCMG_F64) {
    FoldPtrs<double> p;
    for (int k = 0; k < 7; k++) p.A[k] = (double*)get_field(c, it->second.fields[k])->d;
    p.b = (double*)fb->d;
    prof_mark(c, K_BLAS1, stream, true);
    e = launch_fold_boundary<double>(p, g, d_code, c->d_bcval, stream);
    prof_mark(c, K_BLAS1, stream, false);
  } else {
    FoldPtrs<float> p;
    for (int k = 0; k < 7; k++) p.A[k] = (float*)get_field(c, it->second.fields[k])->d;
    p.b = (float*)fb->d;
    prof_mark(c, K_BLAS1, stream, true);
    e = launch_fold_boundary<float>(p, g, d_code, c->d_bcval, stream);
    prof_mark(c, K_BLAS1, stream, false);
  }
  c->launches += 3;
  if (e != cudaSuccess)
    rc = fail(c, BCMG_CUDA_ERROR, "launch failed: %s (%s:%d)", cudaGetErrorString(e), __FILE__,
              __LINE__);
  // the host table must outlive the copy: it is pageable and local
  cudaFreeAsync(d_code, stream);
  cudaError_t se = cudaStreamSynchronize(stream);
  if (!rc && se != cudaSuccess)
    rc = fail(c, BCMG_CUDA_ERROR, "fold: %s", cudaGetErrorString(se));
  return rc;
}

extern "C++" {
template <typename T>
static int make_op(bcmg_ctx c, int opid, const Field& like, Op<T>* out) {
  auto it = c->ops.find(opid);
  if (it == c->ops.end()) return fail(c, BCMG_USAGE, "unknown operator %d", opid);
  out->cc = it->second.d_cc;
  out->cf8 = sizeof(T) == 4 ? (const T*)(const void*)it->second.d_jc32
                            : (const T*)(const void*)it->second.d_jc64;
  for (int k = 0; k < 7; k++) out->A[k] = nullptr;
  if (!out->cc) {
    for (int k = 0; k < 7; k++) {
      Field* f = get_field(c, it->second.fields[k]);
      if (!f) return fail(c, BCMG_USAGE, "operator %d lost a coefficient field", opid);
      if (f->dtype != like.dtype || f->vc != like.vc)
        return fail(c, BCMG_USAGE, "operator coefficients differ from the vector's dtype/vc");
      out->A[k] = (const T*)f->d;
    }
  }
  return BCMG_SUCCESS;
}

}  // extern "C++"

static bool same_shape(const Field* a, const Field* b) {
  return a && b && a->dtype == b->dtype && a->vc == b->vc;
}

static int jacobi_sweep(bcmg_ctx c, int op, Field& x1, Field& x0, Field& b, double omega,
                        cudaStream_t st) {
  Geom g = geom_of(c, x0);
  if (x0.dtype == BCMG_F64) {
    Op<double> o;
    int rc = make_op(c, op, x0, &o);
    if (rc) return rc;
    LAUNCH(c, K_JACOBI, st, launch_jacobi<double>((double*)x1.d, (const double*)x0.d, (const double*)b.d, o, g,
                                    omega, st));
  } else {
    Op<float> o;
    int rc = make_op(c, op, x0, &o);
    if (rc) return rc;
    LAUNCH(c, K_JACOBI, st, launch_jacobi<float>((float*)x1.d, (const float*)x0.d, (const float*)b.d, o, g,
                                   (float)omega, st));
  }
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_jacobi_sweep(bcmg_ctx c, int op, int x1, int x0, int b, double omega, void* st) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {x1, x0, b}, "bcmg_jacobi_sweep")) return rc_host;
  Field *f1 = get_field(c, x1), *f0 = get_field(c, x0), *fb = get_field(c, b);
  if (!same_shape(f1, f0) || !same_shape(f0, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  return jacobi_sweep(c, op, *f1, *f0, *fb, omega, S(c, st));
}

static int residual(bcmg_ctx c, int op, Field* out, Field& x, Field* b, int mode, cudaStream_t st) {
  Geom g = geom_of(c, x);
  if (x.dtype == BCMG_F64) {
    Op<double> o;
    int rc = make_op(c, op, x, &o);
    if (rc) return rc;
    LAUNCH(c, K_RESIDUAL, st, launch_residual<double>(out ? (double*)out->d : nullptr, (const double*)x.d,
                                      b ? (const double*)b->d : nullptr, o, g, mode,
                                      c->d_partial, st));
  } else {
    Op<float> o;
    int rc = make_op(c, op, x, &o);
    if (rc) return rc;
    LAUNCH(c, K_RESIDUAL, st, launch_residual<float>(out ? (float*)out->d : nullptr, (const float*)x.d,
                                     b ? (const float*)b->d : nullptr, o, g, mode, c->d_partial,
                                     st));
  }
  return BCMG_SUCCESS;
}

// Sum the per-block partials and bring the value to the host.
static int finish_reduce(bcmg_ctx c, double* out, cudaStream_t st) {
  LAUNCH(c, K_DOT, st, launch_reduce_final(c->d_partial, c->nb, c->d_scalar, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->h_scalar, c->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(c, cudaStreamSynchronize(st));
  *out = c->h_scalar[0];
  return BCMG_SUCCESS;
}

static int dot(bcmg_ctx c, Field& x, Field& y, double* out, cudaStream_t st) {
  Geom g = geom_of(c, x);
  if (x.dtype == BCMG_F64)
    LAUNCH(c, K_DOT, st, launch_dot_partial<double>((const double*)x.d, (const double*)y.d, g, c->d_partial, st));
  else
    LAUNCH(c, K_DOT, st, launch_dot_partial<float>((const float*)x.d, (const float*)y.d, g, c->d_partial, st));
  return finish_reduce(c, out, st);
}

BCMG_API int bcmg_calc_ax(bcmg_ctx c, int op, int ax, int x, void* st) {
  if (!c) return BCMG_USAGE;
  Field *fa = get_field(c, ax), *fx = get_field(c, x);
  if (!same_shape(fa, fx)) return fail(c, BCMG_USAGE, "field mismatch");
  return residual(c, op, fa, *fx, nullptr, 0, S(c, st));
}

BCMG_API int bcmg_calc_r(bcmg_ctx c, int op, int r, int x, int b, void* st) {
  if (!c) return BCMG_USAGE;
  Field *fr = get_field(c, r), *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fr, fx) || !same_shape(fx, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  return residual(c, op, fr, *fx, fb, 1, S(c, st));
}

BCMG_API int bcmg_calc_r2(bcmg_ctx c, int op, int x, int b, double* rr, void* st) {
  if (!c || !rr) return BCMG_USAGE;
  Field *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fx, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  int rc = residual(c, op, nullptr, *fx, fb, 2, S(c, st));
  if (rc) return rc;
  return finish_reduce(c, rr, S(c, st));
}

BCMG_API int bcmg_dot(bcmg_ctx c, int x, int y, double* out, void* st) {
  if (!c || !out) return BCMG_USAGE;
  Field *fx = get_field(c, x), *fy = get_field(c, y);
  if (!same_shape(fx, fy)) return fail(c, BCMG_USAGE, "field mismatch");
  return dot(c, *fx, *fy, out, S(c, st));
}

static int blas1(bcmg_ctx c, int kind, Field& z, Field* x, Field* y, double a, double b,
                 cudaStream_t st) {
  Geom g = geom_of(c, z);
  if (z.dtype == BCMG_F64)
    LAUNCH(c, K_BLAS1, st, launch_blas1<double>(kind, (double*)z.d, x ? (const double*)x->d : nullptr,
                                   y ? (const double*)y->d : nullptr, a, b, g, st));
  else
    LAUNCH(c, K_BLAS1, st, launch_blas1<float>(kind, (float*)z.d, x ? (const float*)x->d : nullptr,
                                  y ? (const float*)y->d : nullptr, (float)a, (float)b, g, st));
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_axpy(bcmg_ctx c, int y, int x, double a, void* st) {
  if (!c) return BCMG_USAGE;
  Field *fy = get_field(c, y), *fx = get_field(c, x);
  if (!same_shape(fy, fx)) return fail(c, BCMG_USAGE, "field mismatch");
  return blas1(c, 0, *fy, fx, nullptr, a, 0, S(c, st));
}
BCMG_API int bcmg_xpay(bcmg_ctx c, int y, int x, double a, void* st) {
  if (!c) return BCMG_USAGE;
  Field *fy = get_field(c, y), *fx = get_field(c, x);
  if (!same_shape(fy, fx)) return fail(c, BCMG_USAGE, "field mismatch");
  return blas1(c, 1, *fy, fx, nullptr, a, 0, S(c, st));
}
BCMG_API int bcmg_axpyz(bcmg_ctx c, int z, int x, int y, double a, void* st) {
  if (!c) return BCMG_USAGE;
  Field *fz = get_field(c, z), *fx = get_field(c, x), *fy = get_field(c, y);
  if (!same_shape(fz, fx) || !same_shape(fx, fy)) return fail(c, BCMG_USAGE, "field mismatch");
  return blas1(c, 2, *fz, fx, fy, a, 0, S(c, st));
}
BCMG_API int bcmg_axpbypz(bcmg_ctx c, int z, int x, int y, double a, double b, void* st) {
  if (!c) return BCMG_USAGE;
  Field *fz = get_field(c, z), *fx = get_field(c, x), *fy = get_field(c, y);
  if (!same_shape(fz, fx) || !same_shape(fx, fy)) return fail(c, BCMG_USAGE, "field mismatch");
  return blas1(c, 3, *fz, fx, fy, a, b, S(c, st));
}

// ---------------------------------------------------------------------------
// IsConverged (ILS3D.h:41-63): 1 converged, 0 not, -1 NaN/Inf.
static int converged(double rr, double bb, double eps, double* res) {
  const double residual = (std::fabs(bb) > 1.17549435e-38) ? std::fabs(rr) / std::fabs(bb)
                                                             : std::fabs(rr);
  *res = residual;
  if (residual <= eps * eps) return 1;
  if (std::isnan(residual) || std::isinf(residual)) return -1;
  return 0;
}

// Fused Jacobi launch x0 -> x1 (sweep + Dirichlet + ghost push, and the
// residual of x0 into the per-block partials when `res`).
// Fused Jacobi launch x0 -> x1 (sweep + ghosts, and the residual of x0 into
// the per-block partials when `res`).  Push form: x1 leaves with every ghost
// updated.  Pull form: launch 0 of a run (seq) reads x0's ghosts as they are,
// later launches pull them from x0's neighbours and the side buffer the
// previous launch wrote; x1's ghosts then need impose() before any other
// reader (finish_fused).
// Fused-Jacobi choice for field x: 1 push form, 2 pull form one CTA per
// block, 3 pull form pipelined.  Forced by the autotuner, then by the user's
// ghost form / shape, then tuned, else by mesh size (small meshes fit one wave
// of CTAs, where the push form has the shortest chain of dependent loads).
enum { kJacPush = 1, kJacPullTile = 2, kJacPullPipe = 3 };
static long jacobi_key(int dtype, int n, int vc) { return ((long)dtype * 64 + n) * 8 + vc; }
static int jacobi_choice(bcmg_ctx c, const Field& x) {
  if (c->nx == 32) return kJacPush;  // the only fused form of 32^3 blocks
  if (c->jacobi_force) return c->jacobi_force;
  if (c->ghost_form == BCMG_GHOST_PUSH) return kJacPush;
  if (c->jacobi_shape) return c->jacobi_shape == kJacobiPipe ? kJacPullPipe : kJacPullTile;
  auto it = c->jacobi_tuned.find(jacobi_key(x.dtype, c->nx, x.vc));
  if (it != c->jacobi_tuned.end() && (c->ghost_form == BCMG_GHOST_AUTO || it->second != kJacPush))
    return it->second;
  if (c->ghost_form == BCMG_GHOST_PULL) return kJacPullTile;
  return c->nb <= 1024 ? kJacPush : kJacPullTile;
}

// pre (with zero_x0, 32^3 streamed pass): the vector update that makes b,
// fused into the launch (JacPre): kind, r, q and the segments' scalars.
struct PreArgs {
  int kind;
  const Field* r;
  const Field* q;
  KSegs segs;
};

static int jacobi_fused(bcmg_ctx c, const OpRec& o, const Field& x0, const Field& x1,
                        const Field& b, double omega, bool homogeneous, bool res, int seq,
                        int choice, cudaStream_t st, bool zero_x0 = false,
                        const PreArgs* pre = nullptr) {
  Geom g = geom_of(c, x0);
  BlockBc bc{c->bctype.empty() ? nullptr : c->d_bctype,
             homogeneous ? c->d_bczero : c->d_bcval, c->bcform == BCMG_DIRICHLET_BCX ? 1 : 0,
             homogeneous ? c->d_bczero2f : c->d_bcv2f};
  if (choice != kJacPush) {
    int rc = ensure_side(c, dsize(x0.dtype));
    if (rc) return rc;
  }
  PushTable push = push_table(c, seq);
  const int mode = choice == kJacPush ? (zero_x0 ? kGhostPushZero : kGhostPush)
                   : seq == 0 ? kGhostAsIs : kGhostPull;
  const int shape = choice == kJacPullPipe ? kJacobiPipe : kJacobiTile;
  double* part = res ? c->d_partial : nullptr;
  if (x0.dtype == BCMG_F64) {
    JacPre<double> jp{pre ? pre->kind : kPreNone, pre ? (const double*)pre->r->d : nullptr,
                      pre && pre->q ? (const double*)pre->q->d : nullptr,
                      pre ? pre->segs : KSegs{}};
    LAUNCH(c, K_JACOBI, st, launch_jacobi_fused<double>((const double*)x0.d, (double*)x1.d,
                                                         (const double*)b.d, g, o.d_jc64, omega,
                                                         bc, push, mode, shape, part, c->d_err,
                                                         pre ? &jp : nullptr, st));
  } else {
    JacPre<float> jp{pre ? pre->kind : kPreNone, pre ? (const float*)pre->r->d : nullptr,
                     pre && pre->q ? (const float*)pre->q->d : nullptr,
                     pre ? pre->segs : KSegs{}};
    LAUNCH(c, K_JACOBI, st, launch_jacobi_fused<float>((const float*)x0.d, (float*)x1.d,
                                                        (const float*)b.d, g, o.d_jc32,
                                                        (float)omega, bc, push, mode, shape, part,
                                                        c->d_err, pre ? &jp : nullptr, st));
  }
  return BCMG_SUCCESS;
}

// Ghost update closing a run of pull-form fused launches on x.
static int finish_fused(bcmg_ctx c, Field& x, bool homogeneous, int choice, cudaStream_t st) {
  if (choice == kJacPush) return BCMG_SUCCESS;
  return impose(c, x, homogeneous, st);
}

// Whether the fused Jacobi kernel covers this operator and field.
static bool jacobi_fusable(bcmg_ctx c, int op, const Field& x) {
  auto it = c->ops.find(op);
  if (c->no_fusion || c->bc_conflict || c->has_neumann || it == c->ops.end() || !it->second.d_cc)
    return false;
  if (c->nx != c->ny || c->ny != c->nz || (x.vc != 1 && x.vc != 2)) return false;
  if (c->nx == 32) return true;  // push form, no staging
  if (c->nx != 8 && c->nx != 16) return false;
  const size_t es = dsize(x.dtype), n = c->nx, lx = n + 2 * x.vc;
  return 16 + (lx * lx * lx + n * lx * lx) * es <= kSorMaxSmem;
}

BCMG_API int bcmg_jacobi_run(bcmg_ctx c, int op, int x, int b, double omega, int iters,
                             int use_graph, void* st) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {x, b}, "bcmg_jacobi_run")) return rc_host;
  Field *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fx, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  if (iters < 0) return fail(c, BCMG_USAGE, "iters < 0");
  cudaStream_t stream = S(c, st);
  int wid, rc;
  if ((rc = work_field(c, fx->dtype, fx->vc, 32, &wid))) return rc;
  fx = get_field(c, x); fb = get_field(c, b);
  Field* fw = get_field(c, wid);
  if (!jacobi_fusable(c, op, *fx)) {
    // separate sweep + ghost update launches, the reference's order, ping-pong
    // between x and a work copy that starts equal to x (cells that neither the
    // sweep nor the ghost update writes keep x's values in both)
    CUDA_TRY(c, cudaMemcpyAsync(fw->d, fx->d, fx->bytes, cudaMemcpyDeviceToDevice, stream));
    Field* A = fx;
    Field* B = fw;
    for (int k = 0; k < iters; k++) {
      if ((rc = jacobi_sweep(c, op, *B, *A, *fb, omega, stream))) return rc;
      if ((rc = impose(c, *B, false, stream))) return rc;
      std::swap(A, B);
    }
    if (A != fx)
      CUDA_TRY(c, cudaMemcpyAsync(fx->d, A->d, fx->bytes, cudaMemcpyDeviceToDevice, stream));
    return BCMG_SUCCESS;
  }
  const OpRec& o = c->ops[op];
  const int choice = jacobi_choice(c, *fx);
  auto body = [&]() -> int {
    // the work copy starts equal to x: cells no launch writes agree in both
    CUDA_TRY(c, cudaMemcpyAsync(fw->d, fx->d, fx->bytes, cudaMemcpyDeviceToDevice, stream));
    Field* A = fx;
    Field* B = fw;
    for (int k = 0; k < iters; k++) {
      int r2 = jacobi_fused(c, o, *A, *B, *fb, omega, false, false, k, choice, stream);
      if (r2) return r2;
      std::swap(A, B);
    }
    if (iters > 0) {
      int r2 = finish_fused(c, *A, false, choice, stream);
      if (r2) return r2;
    }
    if (A != fx)
      CUDA_TRY(c, cudaMemcpyAsync(fx->d, A->d, fx->bytes, cudaMemcpyDeviceToDevice, stream));
    return BCMG_SUCCESS;
  };
  if (!use_graph || c->profiling) return body();
  // One CUDA graph per (x, b, work, op, iters, omega): replays the whole run.
  const GraphKey key{fx->d, fb->d, fw->d, op, iters, omega, choice};
  auto it = c->graphs.find(key);
  if (it == c->graphs.end()) {
    if (stream == 0) return fail(c, BCMG_USAGE, "graph capture needs a non-default stream");
    // One eager launch first (into the work copy; x is untouched) so the
    // kernel's one-time attribute setup happens outside the capture.
    if ((rc = jacobi_fused(c, o, *fx, *fw, *fb, omega, false, false, 0, choice, stream)))
      return rc;
    CUDA_TRY(c, cudaStreamSynchronize(stream));
    CUDA_TRY(c, cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = c->launches;
    rc = body();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) return fail(c, BCMG_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(e));
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(c, BCMG_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(e));
    c->graphs[key] = GraphRec{exec, c->launches - l0};
    c->launches = l0;
    it = c->graphs.find(key);
  }
  CUDA_TRY(c, cudaGraphLaunch(it->second.exec, stream));
  c->launches += it->second.kernels;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_autotune_jacobi(bcmg_ctx c, int op, int x, int b, double omega, int iters,
                                  int* best, double* best_us) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {x, b}, "bcmg_autotune_jacobi")) return rc_host;
  Field *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fx, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  if (iters < 1) iters = 1;
  if (!jacobi_fusable(c, op, *fx)) {
    if (best) *best = 0;
    if (best_us) *best_us = 0.0;
    return BCMG_SUCCESS;  // separate launches: nothing to choose
  }
  int tid;
  int rc = work_field(c, fx->dtype, fx->vc, 33, &tid);
  if (rc) return rc;
  fx = get_field(c, x);
  Field* t = get_field(c, tid);
  // per-sweep cost: a run of 2*iters sweeps less a run of iters, so that a
  // run's fixed costs (the closing ghost update of the pull forms, the work
  // copy) do not favour one form in short tuning runs
  cudaEvent_t e0, e1, e2;
  CUDA_TRY(c, cudaEventCreate(&e0));
  CUDA_TRY(c, cudaEventCreate(&e1));
  CUDA_TRY(c, cudaEventCreate(&e2));
  const bool only_push = c->nx == 32;  // 32^3 blocks have the push form alone
  int bv = only_push ? kJacPush : kJacPullTile;
  double bt = 1e300;
  for (int v = kJacPush; v <= kJacPullPipe; v++) {
    if (only_push && v != kJacPush) continue;
    if (!only_push && v == kJacPush && c->ghost_form == BCMG_GHOST_PULL) continue;
    if (v != kJacPush && c->ghost_form == BCMG_GHOST_PUSH) continue;
    c->jacobi_force = v;
    CUDA_TRY(c, cudaMemcpyAsync(t->d, fx->d, fx->bytes, cudaMemcpyDeviceToDevice, c->stream));
    rc = bcmg_jacobi_run(c, op, tid, b, omega, 2, 0, c->stream);  // warm-up
    if (rc == BCMG_SUCCESS) {
      cudaEventRecord(e0, c->stream);
      rc = bcmg_jacobi_run(c, op, tid, b, omega, iters, 0, c->stream);
      cudaEventRecord(e1, c->stream);
    }
    if (rc == BCMG_SUCCESS) {
      rc = bcmg_jacobi_run(c, op, tid, b, omega, 2 * iters, 0, c->stream);
      cudaEventRecord(e2, c->stream);
    }
    c->jacobi_force = 0;
    if (rc != BCMG_SUCCESS) break;
    CUDA_TRY(c, cudaEventSynchronize(e2));
    float m1 = 0.f, m2 = 0.f;
    cudaEventElapsedTime(&m1, e0, e1);
    cudaEventElapsedTime(&m2, e1, e2);
    const double ms = m2 - m1 > 0.f ? (double)(m2 - m1) : (double)m2 / 2;
    if (ms < bt) { bt = ms; bv = v; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  if (rc != BCMG_SUCCESS) return rc;
  c->jacobi_tuned[jacobi_key(fx->dtype, c->nx, fx->vc)] = bv;
  if (best) *best = bv;
  if (best_us) *best_us = bt * 1e3 / iters;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_jacobi_solve(bcmg_ctx c, int op, int x, int b, double omega, int max_iter,
                               double eps, bcmg_solve_info* info, void* st) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {x, b}, "bcmg_jacobi_solve")) return rc_host;
  if (c->nseg > 1)
    return fail(c, BCMG_USAGE, "bcmg_jacobi_solve solves one system; the mesh has %d segments",
                c->nseg);
  Field *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fx, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  cudaStream_t stream = S(c, st);
  int wid;
  int rc = work_field(c, fx->dtype, fx->vc, 0, &wid);
  if (rc) return rc;
  fx = get_field(c, x); fb = get_field(c, b);
  Field* fw = get_field(c, wid);
  double bb, rr = 0, res = 0;
  rc = dot(c, *fb, *fb, &bb, stream);
  if (rc) return rc;
  int count, status = BCMG_NOT_CONVERGED;
  if (jacobi_fusable(c, op, *fx)) {
    // Launch k writes x_k (ghosts complete) into the other buffer and the
    // residual of its input x_{k-1}; the reference tests x_{k-1} right after
    // producing it, so the same test runs one launch later on the same values.
    const OpRec& o = c->ops[op];
    const int choice = jacobi_choice(c, *fx);
    CUDA_TRY(c, cudaMemcpyAsync(fw->d, fx->d, fx->bytes, cudaMemcpyDeviceToDevice, stream));
    bool done = false;
    for (count = 1; count <= max_iter; ++count) {
      if ((rc = jacobi_fused(c, o, *fx, *fw, *fb, omega, false, true, count - 1, choice,
                             stream)))
        return rc;
      if ((rc = finish_reduce(c, &rr, stream))) return rc;
      if (count >= 2) {
        const int cv = converged(rr, bb, eps, &res);
        if (cv != 0) {
          status = cv > 0 ? BCMG_SUCCESS : BCMG_DIVERGED;
          count -= 1;  // the answer is the launch's input, still in x
          done = true;
          break;
        }
      }
      std::swap(fx->d, fw->d);  // LSSwap
    }
    if ((rc = finish_fused(c, *fx, false, choice, stream))) return rc;
    if (!done) {
      count = max_iter;
      if ((rc = residual(c, op, nullptr, *fx, fb, 2, stream))) return rc;
      if ((rc = finish_reduce(c, &rr, stream))) return rc;
      const int cv = converged(rr, bb, eps, &res);
      if (cv > 0) status = BCMG_SUCCESS;
      if (cv < 0) status = BCMG_DIVERGED;
    }
    CUDA_TRY(c, cudaStreamSynchronize(stream));
    if ((rc = take_dev_err(c, "Jacobi"))) return rc;
    if (info) {
      info->iterations = count;
      info->residual = res;
      info->status = status;
      info->refinements = 0;
      info->true_residual = std::sqrt(res);
      info->fp64_iterations = 0;
    }
    return status == BCMG_DIVERGED ? BCMG_DIVERGED : BCMG_SUCCESS;
  }
  for (count = 1; count <= max_iter; ++count) {
    rc = jacobi_sweep(c, op, *fw, *fx, *fb, omega, stream);
    if (rc) return rc;
    std::swap(fx->d, fw->d);  // LSSwap
    if ((rc = impose(c, *fx, false, stream))) return rc;
    if ((rc = residual(c, op, nullptr, *fx, fb, 2, stream))) return rc;
    if ((rc = finish_reduce(c, &rr, stream))) return rc;
    int cv = converged(rr, bb, eps, &res);
    if (cv > 0) { status = BCMG_SUCCESS; break; }
    if (cv < 0) { status = BCMG_DIVERGED; break; }
  }
  if (count > max_iter) count = max_iter;
  if ((rc = impose(c, *fx, false, stream))) return rc;
  CUDA_TRY(c, cudaStreamSynchronize(stream));
  if ((rc = take_dev_err(c, "Jacobi"))) return rc;
  if (info) {
    info->iterations = count;
    info->residual = res;
    info->status = status;
    info->refinements = 0;
    info->true_residual = std::sqrt(res);
    info->fp64_iterations = 0;
  }
  return status == BCMG_DIVERGED ? BCMG_DIVERGED : BCMG_SUCCESS;
}

// Jacobi_PreConditioner (ILS3D.h:452-475) on homogeneous boundary values.
// n Jacobi passes (sweep, swap, homogeneous ghosts) of the preconditioner.
// Where the push-form fused sweep applies and no face keeps unupdated ghosts
// (whose values would then come from the input instead of staying as the
// output buffer had them), each pass is one fused launch.
// zero_start: x is zero (ghosts included) before the first pass -- cleared
// here, or, for the 32^3 push-form kernel, taken as zero without a read.
// The zero-start pass of a 32^3 preconditioner can also make its right-hand
// side (PreArgs): the streamed kernels' shapes, fused sweeps.
static bool jacobi_pre_fuses(bcmg_ctx c, int op, const Field& x, int n) {
  return n >= 1 && !c->open_faces && jacobi_fusable(c, op, x) && c->nx == 32 && c->ny == 32 &&
         c->nz == 32 && (x.vc == 1 || x.vc == 2) && plane_stream_enabled();
}

static int jacobi_pre(bcmg_ctx c, int op, Field& x, Field& x0, Field& b, double omega, int n,
                      cudaStream_t st, bool zero_start = false, const PreArgs* pre = nullptr) {
  const bool fused = !c->open_faces && jacobi_fusable(c, op, x);
  const bool zero_kernel = zero_start && fused && c->nx == 32 && n >= 1;
  if (pre && !(zero_kernel && jacobi_pre_fuses(c, op, x, n)))
    return fail(c, BCMG_FAILURE, "internal: preconditioner pass cannot make its right-hand side");
  if (zero_start && !zero_kernel) CUDA_TRY(c, cudaMemsetAsync(x.d, 0, x.bytes, st));
  for (int k = 0; k < n; k++) {
    int rc;
    if (fused) {
      rc = jacobi_fused(c, c->ops[op], x, x0, b, omega, true, false, 0, kJacPush, st,
                        zero_kernel && k == 0, k == 0 ? pre : nullptr);
      if (rc) return rc;
      std::swap(x.d, x0.d);
      continue;
    }
    rc = jacobi_sweep(c, op, x0, x, b, omega, st);
    if (rc) return rc;
    std::swap(x.d, x0.d);
    if ((rc = impose(c, x, true, st))) return rc;
  }
  return BCMG_SUCCESS;
}

// Scratch of the device-resident BiCGSTAB: two FP64 partial sums per block
// and `nseg` scalar records (device, and a pinned host mirror).
static int kr_scratch(bcmg_ctx c, int nseg) {
  if (c->kpart_nb < c->nb) {
    cudaFree(c->d_kpart);
    c->d_kpart = nullptr;
    c->kpart_nb = 0;
    CUDA_TRY(c, cudaMalloc(&c->d_kpart, (size_t)2 * c->nb * sizeof(double)));
    c->kpart_nb = c->nb;
  }
  if (c->kseg_cap < nseg) {
    cudaFree(c->d_kseg);
    cudaFreeHost(c->h_kseg);
    c->d_kseg = nullptr;
    c->h_kseg = nullptr;
    c->kseg_cap = 0;
    CUDA_TRY(c, cudaMalloc(&c->d_kseg, (size_t)nseg * sizeof(KSeg)));
    CUDA_TRY(c, cudaMallocHost(&c->h_kseg, (size_t)nseg * sizeof(KSeg)));
    c->kseg_cap = nseg;
  }
  return BCMG_SUCCESS;
}

// The vectors of one BiCGSTAB solve (ILS3D.h:663-844): x, b and the nine
// work fields r, r0, p, p^, q^, s, s^, t^, x0, plus x's best copy.
struct KrVecs {
  Field *x, *b, *r, *r0, *p, *p_, *q_, *s, *s_, *t_, *x0, *xbest;
};

}  // extern "C" (templates below)

// One BiCGSTAB iteration, queued without a host round trip: its scalars
// come from and go to the segments' records on the device.
template <typename T>
static int kr_iteration(bcmg_ctx c, int op, const KrVecs& v, const Op<T>& o, KSegs S,
                        double omega, int n_pre, int max_iter, double eps2, bool keep_best,
                        bool first, cudaStream_t st) {
  const Geom g = geom_of(c, *v.x);
  double* part = c->d_kpart;
  int rc;
  auto d = [](Field* f) { return (T*)f->d; };
  // 32^3 blocks: p's and s's updates made by their preconditioner's first
  // pass (one launch and one read of p / s fewer each)
  const bool fuse = jacobi_pre_fuses(c, op, *v.p_, n_pre);
  const PreArgs pre_p{first ? kPreCopy : kPreP, v.r, v.q_, S};
  const PreArgs pre_s{kPreS, v.r, v.q_, S};
  if (!fuse) {
    if (first)
      CUDA_TRY(c, cudaMemcpyAsync(v.p->d, v.r->d, v.r->bytes, cudaMemcpyDeviceToDevice, st));
    else
      LAUNCH(c, K_BLAS1, st, launch_kr_p<T>(d(v.p), d(v.r), d(v.q_), g, S, st));
  }
  // ILS3D imposes the boundary condition on p and s (ILS3D.h:741, 774), but
  // nothing here reads their ghosts: the preconditioner reads its right-hand
  // side at the cell only (jacobi_smoother, blas.f90:452-502), and the
  // stencils run on p^ and s^.  Leaving the two ghost updates out changes no
  // value.
  if ((rc = jacobi_pre(c, op, *v.p_, *v.x0, *v.p, omega, n_pre, st, true, fuse ? &pre_p : nullptr)))
    return rc;
  LAUNCH(c, K_RESIDUAL, st, launch_kr_ax<T>(d(v.q_), d(v.p_), o, d(v.r0), 1, g, S, part, c->d_err, st));
  LAUNCH(c, K_DOT, st, launch_kr_scalar(part, c->nb, S, KS_ALPHA, max_iter, eps2, keep_best, st));
  if (!fuse) LAUNCH(c, K_BLAS1, st, launch_kr_s<T>(d(v.s), d(v.r), d(v.q_), g, S, st));
  if ((rc = jacobi_pre(c, op, *v.s_, *v.x0, *v.s, omega, n_pre, st, true, fuse ? &pre_s : nullptr)))
    return rc;
  LAUNCH(c, K_RESIDUAL, st, launch_kr_ax<T>(d(v.t_), d(v.s_), o, d(v.s), 2, g, S, part, c->d_err, st));
  LAUNCH(c, K_DOT, st, launch_kr_scalar(part, c->nb, S, KS_GAMMA, max_iter, eps2, keep_best, st));
  LAUNCH(c, K_BLAS1, st, launch_kr_xr<T>(d(v.x), d(v.r), d(v.p_), d(v.s_), d(v.s), d(v.t_),
                                         d(v.r0), g, S, part, c->d_err, st));
  LAUNCH(c, K_DOT, st, launch_kr_scalar(part, c->nb, S, KS_R, max_iter, eps2, keep_best, st));
  if (keep_best) LAUNCH(c, K_BLAS1, st, launch_kr_best<T>(d(v.xbest), d(v.x), g, S, st));
  return BCMG_SUCCESS;
}

// BiCGSTAB of ILS3D.h:663-844, device-resident, for every segment of the
// mesh at once (one segment: an ordinary solve).  The scalars live on the
// device (krylov.cuh) and the host queues iterations in growing chunks
// (1, 1, 2, 4, ... 16), reading the segments' status back after each chunk;
// iterations queued past a segment's end change nothing of its x or r
// (their vector kernels skip a finished segment).  Direction vectors carry
// homogeneous Dirichlet ghosts, which is the ghost-cell form of the
// reference's boundary-folded matrix (SolverTest/bca.f90:12-42).  keep_best
// (the mixed-precision driver's correction solves): x leaves as the iterate
// with the smallest recursive residual seen, not the last one -- a
// correction is then never one that FP32 round-off blew up at the end.
// active / maxit (host copies, null: every segment, max_iter): the segments
// taking part and their own iteration limits.  info: one record per segment.
template <typename T>
static int bicgstab_dev(bcmg_ctx c, int op, KrVecs v, double omega, int n_pre, int max_iter,
                        double eps, bcmg_solve_info* info, cudaStream_t st, bool keep_best,
                        const std::vector<unsigned char>* active = nullptr,
                        const std::vector<int>* maxit = nullptr,
                        const std::vector<double>* eps_seg = nullptr) {
  int rc;
  Op<T> o;
  const int nseg = c->nseg;
  if ((rc = make_op(c, op, *v.x, &o))) return rc;
  if ((rc = kr_scratch(c, nseg))) return rc;
  if ((rc = seg_buffers(c, nseg))) return rc;
  KSegs S{c->d_kseg, c->d_seg_of, nseg > 1 ? c->d_seg_first : nullptr, nseg, nullptr, nullptr,
          nullptr};
  int limit = max_iter;
  std::vector<double> e2;
  if (eps_seg) {
    e2.resize(nseg);
    for (int q = 0; q < nseg; q++) e2[q] = (*eps_seg)[q] * (*eps_seg)[q];
    CUDA_TRY(c, cudaMemcpyAsync(c->d_segeps2, e2.data(), (size_t)nseg * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    S.seg_eps2 = c->d_segeps2;
  }
  if (active) {
    CUDA_TRY(c, cudaMemcpyAsync(c->d_segflag, active->data(), (size_t)nseg,
                                cudaMemcpyHostToDevice, st));
    S.seg_active = c->d_segflag;
  }
  if (maxit) {
    CUDA_TRY(c, cudaMemcpyAsync(c->d_segmaxit, maxit->data(), (size_t)nseg * sizeof(int),
                                cudaMemcpyHostToDevice, st));
    S.seg_max_iter = c->d_segmaxit;
    limit = 0;
    for (int q = 0; q < nseg; q++) limit = std::max(limit, (*maxit)[q]);
  }
  const Geom g = geom_of(c, *v.x);
  const double eps2 = eps * eps;
  // r = b - A x, r0 = r; b.b and r.r0 (ILS3D.h:690-716)
  if ((rc = residual(c, op, v.r, *v.x, v.b, 1, st))) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(v.r0->d, v.r->d, v.r->bytes, cudaMemcpyDeviceToDevice, st));
  LAUNCH(c, K_DOT, st, launch_kr_dot2<T>((T*)v.b->d, (T*)v.b->d, (T*)v.r->d, (T*)v.r0->d, g,
                                         c->d_kpart, st));
  LAUNCH(c, K_DOT, st, launch_kr_scalar(c->d_kpart, c->nb, S, KS_INIT, max_iter, eps2,
                                        keep_best ? 1 : 0, st));
  auto read_back = [&]() -> int {
    CUDA_TRY(c, cudaMemcpyAsync(c->h_kseg, c->d_kseg, (size_t)nseg * sizeof(KSeg),
                                cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    return BCMG_SUCCESS;
  };
  auto running = [&]() {
    for (int q = 0; q < nseg; q++)
      if (c->h_kseg[q].status == kRunning) return true;
    return false;
  };
  if ((rc = read_back())) return rc;
  int queued = 0, chunk = 1, step = 0;
  while (running()) {
    for (int k = 0; k < chunk; k++, queued++)
      if ((rc = kr_iteration<T>(c, op, v, o, S, omega, n_pre, max_iter, eps2, keep_best,
                                queued == 0, st)))
        return rc;
    if ((rc = read_back())) return rc;
    if (++step >= 2) chunk = std::min(2 * chunk, 16);
    chunk = std::min(chunk, std::max(1, limit - queued));
    if (running() && queued >= limit + 1)
      return fail(c, BCMG_FAILURE, "BiCGSTAB: solve still running after its iteration limit");
  }
  // keep-best segments that ended above their best iterate (limit,
  // breakdown, NaN) take it back
  std::vector<unsigned char> back(nseg, 0);
  bool any_back = false;
  for (int q = 0; q < nseg; q++) {
    const KSeg& h = c->h_kseg[q];
    back[q] = keep_best && h.status != kSkipped && h.status != BCMG_SUCCESS && h.best_saved;
    any_back = any_back || back[q];
  }
  if (any_back) {
    CUDA_TRY(c, cudaMemcpyAsync(c->d_segflag, back.data(), (size_t)nseg, cudaMemcpyHostToDevice,
                                st));
    LAUNCH(c, K_BLAS1, st, launch_kr_seg_copy<T>((T*)v.x->d, (const T*)v.xbest->d, g,
                                                 c->d_seg_of, c->d_segflag, st));
  }
  if ((rc = impose(c, *v.x, false, st))) return rc;
  CUDA_TRY(c, cudaStreamSynchronize(st));
  if ((rc = take_dev_err(c, "BiCGSTAB"))) return rc;
  int worst = BCMG_SUCCESS;
  for (int q = 0; q < nseg; q++) {
    const KSeg& h = c->h_kseg[q];
    if (h.status == kSkipped) continue;
    int status = h.status, count = h.count;
    double res = h.res;
    if (back[q]) {
      res = h.best_rr / h.bb;
      if (status == BCMG_DIVERGED) status = BCMG_NOT_CONVERGED;
    }
    const int lim = maxit ? (*maxit)[q] : max_iter;
    if (count > lim) count = lim;
    if (status == BCMG_DIVERGED) worst = BCMG_DIVERGED;
    if (info) {
      info[q].iterations = count;
      info[q].residual = res;
      info[q].status = status;
      info[q].refinements = 0;
      info[q].true_residual = std::sqrt(res);
      info[q].fp64_iterations = 0;
    }
  }
  return worst;
}

extern "C" {

static int bicgstab_core(bcmg_ctx c, int op, int x, int b, double omega, int n_pre, int max_iter,
                         double eps, bcmg_solve_info* info, cudaStream_t st,
                         bool keep_best = false) {
  Field *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fx, fb)) return fail(c, BCMG_USAGE, "field mismatch");
  if (n_pre < 1) return fail(c, BCMG_USAGE, "n_pre must be >= 1");
  const int dt = fx->dtype, vc = fx->vc;
  int w[9];
  for (int k = 0; k < 9; k++) {
    int rc = work_field(c, dt, vc, 1 + k, &w[k]);
    if (rc) return rc;
  }
  int wbest = -1;
  if (keep_best) {
    int rc2 = work_field(c, dt, vc, 11, &wbest);
    if (rc2) return rc2;
  }
  KrVecs v;
  v.x = get_field(c, x);
  v.b = get_field(c, b);
  v.r = get_field(c, w[0]); v.r0 = get_field(c, w[1]); v.p = get_field(c, w[2]);
  v.p_ = get_field(c, w[3]); v.q_ = get_field(c, w[4]); v.s = get_field(c, w[5]);
  v.s_ = get_field(c, w[6]); v.t_ = get_field(c, w[7]); v.x0 = get_field(c, w[8]);
  v.xbest = keep_best ? get_field(c, wbest) : v.x;
  if (dt == BCMG_F64)
    return bicgstab_dev<double>(c, op, v, omega, n_pre, max_iter, eps, info, st, keep_best);
  return bicgstab_dev<float>(c, op, v, omega, n_pre, max_iter, eps, info, st, keep_best);
}

BCMG_API int bcmg_bicgstab(bcmg_ctx c, int op, int x, int b, double omega, int n_pre,
                           int max_iter, double eps, bcmg_solve_info* info, void* st) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {x, b}, "bcmg_bicgstab")) return rc_host;
  return bicgstab_core(c, op, x, b, omega, n_pre, max_iter, eps, info, S(c, st));
}

}  // extern "C"

// Interior conversion helpers for the mixed-precision driver.
namespace bcmg {
cudaError_t launch_convert_f64_to_f32(float* dst, const double* src, const Geom& g64,
                                      const Geom& g32, cudaStream_t st);
cudaError_t launch_accumulate_f32_into_f64(double* x, const float* d, const Geom& g64,
                                           const Geom& g32, cudaStream_t st);
}  // namespace bcmg

// Per-segment sums of x.y (and u.v) brought to the host: out[2s], out[2s+1].
template <typename T>
static int seg_dots(bcmg_ctx c, Field& x, Field& y, Field& u, Field& v, std::vector<double>* out,
                    cudaStream_t st) {
  int rc;
  if ((rc = kr_scratch(c, c->nseg))) return rc;
  if ((rc = seg_buffers(c, c->nseg))) return rc;
  const Geom g = geom_of(c, x);
  LAUNCH(c, K_DOT, st, launch_kr_dot2<T>((const T*)x.d, (const T*)y.d, (const T*)u.d,
                                         (const T*)v.d, g, c->d_kpart, st));
  KSegs S{c->d_kseg, c->d_seg_of, c->nseg > 1 ? c->d_seg_first : nullptr, c->nseg, nullptr,
          nullptr, nullptr};
  LAUNCH(c, K_DOT, st, launch_kr_segsum(c->d_kpart, c->nb, S, c->d_segsum, st));
  CUDA_TRY(c, cudaMemcpyAsync(c->h_segsum, c->d_segsum, (size_t)2 * c->nseg * sizeof(double),
                              cudaMemcpyDeviceToHost, st));
  CUDA_TRY(c, cudaStreamSynchronize(st));
  out->assign(c->h_segsum, c->h_segsum + 2 * c->nseg);
  return BCMG_SUCCESS;
}

// Per-segment arguments of the segmented kernels to the device.
static int seg_args(bcmg_ctx c, const std::vector<unsigned char>& flag,
                    const std::vector<double>* scale, cudaStream_t st) {
  CUDA_TRY(c, cudaMemcpyAsync(c->d_segflag, flag.data(), flag.size(), cudaMemcpyHostToDevice, st));
  if (scale)
    CUDA_TRY(c, cudaMemcpyAsync(c->d_segscale, scale->data(), scale->size() * sizeof(double),
                                cudaMemcpyHostToDevice, st));
  return BCMG_SUCCESS;
}

extern "C" BCMG_API int bcmg_bicgstab_mixed(bcmg_ctx c, int op, int x, int b, double omega,
                                            int n_pre, int max_inner, double eps_inner,
                                            int max_outer, double eps, bcmg_solve_info* info,
                                            void* stv) {
  if (!c) return BCMG_USAGE;
  if (int rc_host = refuse_host(c, {x, b}, "bcmg_bicgstab_mixed")) return rc_host;
  Field *fx = get_field(c, x), *fb = get_field(c, b);
  if (!same_shape(fx, fb) || fx->dtype != BCMG_F64)
    return fail(c, BCMG_USAGE, "mixed precision needs FP64 x and b of equal shape");
  auto it = c->ops.find(op);
  if (it == c->ops.end() || !it->second.d_cc)
    return fail(c, BCMG_USAGE, "mixed precision needs a per-block constant operator");
  if (n_pre < 1) return fail(c, BCMG_USAGE, "n_pre must be >= 1");
  cudaStream_t st = S(c, stv);
  const int vc = fx->vc, nseg = c->nseg;
  int wr64, wr32, wd32, wprev;
  int rc;
  if ((rc = work_field(c, BCMG_F64, vc, 20, &wr64))) return rc;
  if ((rc = work_field(c, BCMG_F32, vc, 21, &wr32))) return rc;
  if ((rc = work_field(c, BCMG_F32, vc, 22, &wd32))) return rc;
  if ((rc = work_field(c, BCMG_F64, vc, 23, &wprev))) return rc;
  int w32[10];
  for (int k = 0; k < 9; k++)
    if ((rc = work_field(c, BCMG_F32, vc, 1 + k, &w32[k]))) return rc;
  if ((rc = work_field(c, BCMG_F32, vc, 11, &w32[9]))) return rc;
  if ((rc = seg_buffers(c, nseg))) return rc;
  fx = get_field(c, x); fb = get_field(c, b);
  Field *r64 = get_field(c, wr64), *r32 = get_field(c, wr32), *d32 = get_field(c, wd32);
  Field* xprev = get_field(c, wprev);
  const Geom g64 = geom_of(c, *fx), g32 = geom_of(c, *r32);
  // the FP32 correction solve's vectors: d32 for b's place is its unknown,
  // r32 its right-hand side
  KrVecs v32;
  v32.x = d32; v32.b = r32;
  v32.r = get_field(c, w32[0]); v32.r0 = get_field(c, w32[1]); v32.p = get_field(c, w32[2]);
  v32.p_ = get_field(c, w32[3]); v32.q_ = get_field(c, w32[4]); v32.s = get_field(c, w32[5]);
  v32.s_ = get_field(c, w32[6]); v32.t_ = get_field(c, w32[7]); v32.x0 = get_field(c, w32[8]);
  v32.xbest = get_field(c, w32[9]);

  // per-segment refinement state (the single-system flow of earlier
  // versions, run for every segment in lock step)
  struct Mix {
    int status = BCMG_NOT_CONVERGED;
    bool done = false, finish64 = false, have_prev = false;
    double bnorm = 0, rel = 0, prev = 1e300;
    int inner_cap = 0, outer = 0, inner = 0, fp64 = 0;
  };
  std::vector<Mix> m(nseg);
  std::vector<double> sums;
  if ((rc = seg_dots<double>(c, *fb, *fb, *fb, *fb, &sums, st))) return rc;
  for (int q = 0; q < nseg; q++) {
    m[q].bnorm = std::sqrt(sums[2 * q]);
    m[q].inner_cap = max_inner;
  }
  std::vector<unsigned char> flag(nseg), back(nseg), corr(nseg);
  std::vector<double> scale(nseg), eps_q(nseg, eps_inner);
  std::vector<int> cap(nseg);
  std::vector<bcmg_solve_info> in(nseg);
  for (;;) {
    bool any = false;
    for (int q = 0; q < nseg; q++) any = any || !m[q].done;
    if (!any) break;
    if ((rc = impose(c, *fx, false, st))) return rc;
    if ((rc = residual(c, op, r64, *fx, fb, 1, st))) return rc;  // FP64 r = b - A x
    if ((rc = seg_dots<double>(c, *r64, *r64, *r64, *r64, &sums, st))) return rc;
    bool any_back = false, any_corr = false;
    for (int q = 0; q < nseg; q++) {
      Mix& s = m[q];
      back[q] = corr[q] = 0;
      if (s.done) continue;
      const double rr = sums[2 * q];
      s.rel = s.bnorm > 0 ? std::sqrt(rr) / s.bnorm : std::sqrt(rr);
      if (std::isnan(s.rel) || std::isinf(s.rel)) { s.status = BCMG_DIVERGED; s.done = true; continue; }
      if (s.rel <= eps) { s.status = BCMG_SUCCESS; s.done = true; continue; }
      // a refinement that did not reduce the residual: x goes back to
      // before it, and the correction solves restart twice as often
      // (shorter FP32 runs drift less from the true residual) until they
      // are too short
      if (s.rel >= s.prev && s.have_prev) {
        back[q] = 1;
        any_back = true;
        s.have_prev = false;
        s.inner_cap /= 2;
        if (s.inner_cap < 10 || s.outer == max_outer) {
          s.rel = s.prev;
          s.done = true;
          s.finish64 = true;
        } else {
          s.outer++;  // the residual of the restored x, then a shorter correction
        }
        continue;
      }
      if (s.outer == max_outer) { s.done = true; s.finish64 = true; continue; }
      s.prev = s.rel;
      corr[q] = 1;
      any_corr = true;
      scale[q] = 1.0 / std::sqrt(rr);  // the correction problem scaled to a unit residual
      cap[q] = s.inner_cap;
      // a correction need not reduce the residual further than the target
      // asks (with a factor two to spare): the last one is often short
      eps_q[q] = std::max(eps_inner, 0.5 * eps / s.rel);
    }
    if (any_back) {
      if ((rc = seg_args(c, back, nullptr, st))) return rc;
      LAUNCH(c, K_BLAS1, st, launch_kr_seg_copy<double>((double*)fx->d, (const double*)xprev->d,
                                                        g64, c->d_seg_of, c->d_segflag, st));
    }
    if (!any_corr) continue;
    // A d = r / |r| in FP32 for the correcting segments
    if ((rc = seg_args(c, corr, &scale, st))) return rc;
    LAUNCH(c, K_OTHER, st, launch_kr_seg_to32((float*)r32->d, (const double*)r64->d, g32, g64,
                                              c->d_seg_of, c->d_segflag, c->d_segscale, st));
    CUDA_TRY(c, cudaMemsetAsync(d32->d, 0, d32->bytes, st));
    if ((rc = impose(c, *d32, true, st))) return rc;
    rc = bicgstab_dev<float>(c, op, v32, omega, n_pre, max_inner, eps_inner, in.data(), st, true,
                             &corr, &cap, &eps_q);
    if (rc && rc != BCMG_DIVERGED) return rc;
    // segments whose correction diverged before any usable iterate keep x
    // and go to the FP64 finish; the others accumulate |r| d in FP64
    std::vector<unsigned char> acc(nseg, 0);
    bool any_acc = false;
    for (int q = 0; q < nseg; q++) {
      if (!corr[q]) continue;
      Mix& s = m[q];
      s.inner += in[q].iterations;
      if (in[q].status == BCMG_DIVERGED) { s.done = true; s.finish64 = true; continue; }
      acc[q] = 1;
      any_acc = true;
      s.have_prev = true;
      s.outer++;
      scale[q] = 1.0 / scale[q];
    }
    if (any_acc) {
      if ((rc = seg_args(c, acc, &scale, st))) return rc;
      LAUNCH(c, K_BLAS1, st, launch_kr_seg_copy<double>((double*)xprev->d, (const double*)fx->d,
                                                        g64, c->d_seg_of, c->d_segflag, st));
      LAUNCH(c, K_OTHER, st, launch_kr_seg_acc((double*)fx->d, (const float*)d32->d, g32, g64,
                                               c->d_seg_of, c->d_segflag, c->d_segscale, st));
    }
  }
  // the FP32 corrections stalled above the target: the FP64 BiCGSTAB takes
  // over from x for those segments (its work vectors are allocated here, on
  // first need)
  std::vector<unsigned char> fin(nseg, 0);
  bool any_fin = false;
  for (int q = 0; q < nseg; q++) {
    fin[q] = m[q].finish64 && m[q].status == BCMG_NOT_CONVERGED && !std::isnan(m[q].rel);
    any_fin = any_fin || fin[q];
  }
  if (any_fin) {
    int w64[9];
    bool room = true;
    for (int k = 0; k < 9 && room; k++) {
      rc = work_field(c, BCMG_F64, vc, 1 + k, &w64[k]);
      if (rc == BCMG_MEMORY) room = false;  // the FP32-refined x stands
      else if (rc) return rc;
    }
    if (room) {
      KrVecs v64;
      v64.x = get_field(c, x); v64.b = get_field(c, b);
      v64.r = get_field(c, w64[0]); v64.r0 = get_field(c, w64[1]); v64.p = get_field(c, w64[2]);
      v64.p_ = get_field(c, w64[3]); v64.q_ = get_field(c, w64[4]); v64.s = get_field(c, w64[5]);
      v64.s_ = get_field(c, w64[6]); v64.t_ = get_field(c, w64[7]); v64.x0 = get_field(c, w64[8]);
      v64.xbest = v64.x;
      std::vector<int> cap64(nseg, std::max(1, max_outer) * max_inner);
      rc = bicgstab_dev<double>(c, op, v64, omega, n_pre, cap64[0], eps, in.data(), st, false,
                                &fin, &cap64);
      if (rc && rc != BCMG_DIVERGED) return rc;
      fx = get_field(c, x); fb = get_field(c, b); r64 = get_field(c, wr64);
      if ((rc = impose(c, *fx, false, st))) return rc;
      if ((rc = residual(c, op, r64, *fx, fb, 1, st))) return rc;
      if ((rc = seg_dots<double>(c, *r64, *r64, *r64, *r64, &sums, st))) return rc;
      for (int q = 0; q < nseg; q++) {
        if (!fin[q]) continue;
        Mix& s = m[q];
        s.fp64 = in[q].iterations;
        s.inner += in[q].iterations;
        const double rr = sums[2 * q];
        s.rel = s.bnorm > 0 ? std::sqrt(rr) / s.bnorm : std::sqrt(rr);
        s.status = s.rel <= eps ? BCMG_SUCCESS
                   : in[q].status == BCMG_DIVERGED ? BCMG_DIVERGED : BCMG_NOT_CONVERGED;
      }
    }
  }
  fx = get_field(c, x);
  if ((rc = impose(c, *fx, false, st))) return rc;
  CUDA_TRY(c, cudaStreamSynchronize(st));
  int worst = BCMG_SUCCESS;
  for (int q = 0; q < nseg; q++) {
    if (m[q].status == BCMG_DIVERGED) worst = BCMG_DIVERGED;
    if (info) {
      info[q].iterations = m[q].inner;
      info[q].residual = m[q].rel * m[q].rel;
      info[q].status = m[q].status;
      info[q].refinements = m[q].outer;
      info[q].true_residual = m[q].rel;
      info[q].fp64_iterations = m[q].fp64;
    }
  }
  return worst;
}

