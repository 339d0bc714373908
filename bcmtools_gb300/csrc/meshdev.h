// meshdev.h -- device-side mesh set-up: the octree's leaves, its 2:1
// balance, the neighbour table and the ghost-update face tables built on
// the GPU (mesh_dev.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "bcmg.h"
#include "common.cuh"
#include "kernels.h"

namespace bcmg {

// Face tables of one block set, in device memory owned by the caller
// (stream-ordered allocations on the set-up's stream; cudaFree releases
// them): the ghost-update entries in 12 categories (kind x axis), the push
// table (entries by source block), the faces' ghost sources, the F2C entries
// by source block and the per-block descriptors of the pull form.
struct FaceTables {
  VcTask* tasks = nullptr;
  int ntasks = 0;
  int cat_start[12] = {}, cat_count[12] = {};
  int* push_ptr = nullptr;
  VcTask* push_tasks = nullptr;
  unsigned char* fed = nullptr;
  FaceIn* facein = nullptr;
  BlockInfo* binfo = nullptr;
  VcTask* out_tasks = nullptr;
  int ghost_slots = 0;
  bool pull_ok = true, open_faces = false, bc_conflict = false, has_neumann = false;
};

// The face tables of nb blocks from the neighbour table (device arrays:
// ld[nb*6], id[nb*24], sf[nb*6]) and the faces' boundary types (device
// bctype[nb*6] or null; bcform the Dirichlet ghost form).  Entry order, side
// slots and tables as BlockManager's face lists give them: categories in
// kind-major, axis-minor order, each in (block, face, subface) order.
cudaError_t build_face_tables(int nb, const int* ld, const int* id, const int* sf,
                              const int* bctype, int bcform, FaceTables* out, cudaStream_t st);

// A block set on the device: leaf pedigrees in block order and the
// neighbour table (as bcmg_octree_neighbors gives it), device arrays owned by
// the caller (stream-ordered allocations, released by mesh_free).
struct MeshDev {
  int nb = 0;
  uint64_t* peds = nullptr;
  int* ld = nullptr;
  int* id = nullptr;
  int* sf = nullptr;
  int* outer = nullptr;
};

// The octree of divider `div` over `rg` (points of a BALLS divider in host
// memory), 2:1 balanced when div.balance, active leaves in Z order, with
// their neighbour table.  BCMG_FAILURE when a level difference across a face
// exceeds one (unbalanced trees), BCMG_USAGE for invalid arguments.
int mesh_from_divider(const bcmg_rootgrid& rg, const bcmg_divider& div, MeshDev* out,
                      cudaStream_t st, const char** why);
// Blocks = the listed leaves (host array) in list order; the regions the
// list leaves out are inactive.  balance: first refine the listed set 2:1
// (refined leaves replace their parents; the block order is then Z order).
int mesh_from_pedigrees(const bcmg_rootgrid& rg, const uint64_t* peds, int n, bool balance,
                        MeshDev* out, cudaStream_t st, const char** why);
void mesh_free(MeshDev* m, cudaStream_t st);

}  // namespace bcmg
