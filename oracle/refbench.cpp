// refbench.cpp -- times the reference's own OpenMP CPU path of the red-black
// SOR benchmark: the examples/sor2 Solver's calcSorInBlock and Dirichlet
// ghost code (its Solver.cpp, compiled from the reference sources) with the
// reference BlockManager's ghost update through Scalar3DUpdater<double>, on
// a mesh given as a pedigree list (BCMOctree(RootGrid*, pedigrees),
// Utils/src/BCMOctree.cpp:66-96).  TEST AND BENCHMARK INFRASTRUCTURE ONLY:
// built by oracle/Makefile into oracle/_ref/, never part of the library.
//
//   refbench <in> <threads> <warmup> <iters> <out>
//
// <in> (little endian): int32 rx, ry, rz, n, vc, nb; double root_length,
// omega; uint64 pedigree[nb]; then nb packed bricks of (n+2vc)^3 doubles, the
// source term s of every block (in pedigree-list order).
// <out>: double seconds of the timed iterations; int32 nb; then per block of
// the reference's block order its uint64 pedigree and the final brick of f.
//
// One iteration is what sor2's Solver::run does per outer step
// (examples/sor2/Solver.cpp:77-133) with nLoopInner = 1: for every block
// calcSorInBlock (both colours) and setBoundaryConditionInBlock, then
// beginUpdateVC, setBoundaryCondition, endUpdateVC.  The one difference is
// the source term: sor2 recomputes its sine source into one work brick per
// block and step (Solver::setSource, :383-405); here every block keeps its
// own source brick, as the GPU benchmark does, so the timed loop is the
// sweep and the ghost update alone.  Solver's sweep and boundary members are
// private; the driver opens them with a macro around the header only.
#include <omp.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "BCMTools.h"
#include "BCMOctree.h"
#include "Block.h"
#include "BlockFactory.h"
#include "BlockManager.h"
#include "BoundaryConditionSetterBase.h"
#include "BoundaryInfo.h"
#include "Config.h"
#include "Partition.h"
#include "RootGrid.h"
#include "Scalar3D.h"
#include "Scalar3DUpdater.h"
#define private public
#include "Solver.h"
#undef private

// Dirichlet 0 on every outer face, as sor2's BoundaryConditionSetter does
// (examples/sor2/BoundaryConditionSetter.h:37-49).
class OuterDirichlet : public BoundaryConditionSetterBase {
 public:
  BoundaryInfo* operator()(const Node* node, const BCMOctree* tree) {
    BoundaryInfo* bi = new BoundaryInfo[NUM_FACE];
    for (int i = 0; i < NUM_FACE; i++) {
      if (tree->checkOnOuterBoundary(node, Face(i))) {
        bi[i].setType(BoundaryInfo::DIRICHLET);
        bi[i].setID(0);
      }
    }
    return bi;
  }
};

template <typename V>
static bool rd(FILE* fp, V* v, size_t n) { return fread(v, sizeof(V), n, fp) == n; }

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: refbench <in> <threads> <warmup> <iters> <out>\n");
    return 2;
  }
  const int threads = atoi(argv[2]), warm = atoi(argv[3]), iters = atoi(argv[4]);
  FILE* fp = fopen(argv[1], "rb");
  if (!fp) return 3;
  int hdr[6];
  double rl_om[2];
  if (!rd(fp, hdr, 6) || !rd(fp, rl_om, 2)) return 3;
  const int rx = hdr[0], ry = hdr[1], rz = hdr[2], n = hdr[3], vc = hdr[4], nb = hdr[5];
  std::vector<uint64_t> ped_in(nb);
  if (!rd(fp, ped_in.data(), nb)) return 3;
  const int n0 = n + 2 * vc;
  const size_t bsz = (size_t)n0 * n0 * n0;
  std::vector<double> src((size_t)nb * bsz);
  if (!rd(fp, src.data(), src.size())) return 3;
  fclose(fp);
  omp_set_num_threads(threads);

  RootGrid* root = new RootGrid(rx, ry, rz);
  std::vector<Pedigree> peds(nb);
  for (int b = 0; b < nb; b++) peds[b].deserialize(&ped_in[b]);
  BCMOctree* tree = new BCMOctree(root, peds);
  const int nl = tree->getNumLeafNode();
  if (nl != nb) return 4;
  std::vector<Node*>& leaves = tree->getLeafNodeArray();
  Partition* part = new Partition(1, nl);
  OuterDirichlet* bcs = new OuterDirichlet;
  // BlockFactory keeps references to its origin and size arguments
  // (Utils/include/BlockFactory.h), so they must outlive it
  const Vec3r rootOrigin(0.0, 0.0, 0.0);
  const Vec3i size(n, n, n);
  BlockFactory factory(tree, part, bcs, rootOrigin, rl_om[0], size);
  BlockManager& bm = BlockManager::getInstance();
  std::vector<uint64_t> ped_out(nl);
  for (int id = 0; id < nl; id++) {
    bm.registerBlock(factory.makeBlock(leaves[id]));
    leaves[id]->getPedigree().serialize(&ped_out[id]);
  }
  bm.endRegisterBlock();

  // sor2's Solver on this mesh (its constructor registers f with the
  // Scalar3DUpdater<double> and prepares its ghost update).  The Config is
  // never destroyed: ConfigBase's constructor leaves its ConfigFile pointer
  // unset and its destructor deletes it (Utils/src/ConfigBase.cpp:24-32),
  // which only load() makes safe.
  Config& conf = *new Config;
  conf.minLevel = 0;
  conf.maxLevel = 0;
  conf.nLoopInner = 1;
  conf.nLoopOuter = 1;
  conf.omega = rl_om[1];
  conf.separate = false;
  conf.size = n;
  conf.vc = vc;
  conf.verbose = false;
  std::vector<double> boundaryValue(1, 0.0);
  Solver solver(conf, boundaryValue);
  const int id_f = 0;  // the Solver's data class, the first one registered
  const int id_s = bm.setDataClass<Scalar3D<double> >(vc);

  // f = 0 with its ghosts set; s from the input, matched by pedigree
  for (int id = 0; id < nl; id++) {
    int src_b = -1;
    for (int b = 0; b < nb && src_b < 0; b++)
      if (ped_in[b] == ped_out[id]) src_b = b;
    if (src_b < 0) return 5;
    Scalar3D<double>* f = dynamic_cast<Scalar3D<double>*>(bm.getBlock(id)->getDataClass(id_f));
    Scalar3D<double>* s = dynamic_cast<Scalar3D<double>*>(bm.getBlock(id)->getDataClass(id_s));
    double* fd = f->getData();
    double* sd = s->getData();
    for (size_t e = 0; e < bsz; e++) {
      fd[e] = 0.0;
      sd[e] = src[(size_t)src_b * bsz + e];
    }
  }
  bm.beginUpdateVC(id_f);
  solver.setBoundaryCondition();
  bm.endUpdateVC(id_f);

  const double omega = rl_om[1];
  auto iterate = [&]() {
    for (int id = 0; id < bm.getNumBlock(); ++id) {
      Block* block = dynamic_cast<Block*>(bm.getBlock(id));
      Scalar3D<double>* f = dynamic_cast<Scalar3D<double>*>(block->getDataClass(id_f));
      Scalar3D<double>* s = dynamic_cast<Scalar3D<double>*>(block->getDataClass(id_s));
      double* fData = f->getData();
      const double* sData = s->getData();
      Index3DS fIndex = f->getIndex();
      const BoundaryInfo* boundaryInfo = block->getBoundaryInfo();
      const Vec3d& cellSize = block->getCellSize();
      double cx = 1.0 / (cellSize.x * cellSize.x);
      double cy = 1.0 / (cellSize.y * cellSize.y);
      double cz = 1.0 / (cellSize.z * cellSize.z);
      double c = 1.0 / (2.0 * (cx + cy + cz));
      solver.calcSorInBlock(n, n, n, fData, sData, fIndex, omega, c, cx, cy, cz);
      solver.setBoundaryConditionInBlock(n, n, n, fData, fIndex, boundaryInfo);
    }
    bm.beginUpdateVC(id_f);
    solver.setBoundaryCondition();
    bm.endUpdateVC(id_f);
  };
  for (int it = 0; it < warm; it++) iterate();
  auto t0 = std::chrono::steady_clock::now();
  for (int it = 0; it < iters; it++) iterate();
  auto t1 = std::chrono::steady_clock::now();
  const double sec = std::chrono::duration<double>(t1 - t0).count();

  FILE* out = fopen(argv[5], "wb");
  if (!out) return 6;
  fwrite(&sec, 8, 1, out);
  fwrite(&nl, 4, 1, out);
  for (int id = 0; id < nl; id++) {
    Scalar3D<double>* f = dynamic_cast<Scalar3D<double>*>(bm.getBlock(id)->getDataClass(id_f));
    fwrite(&ped_out[id], 8, 1, out);
    fwrite(f->getData(), 8, bsz, out);
  }
  fclose(out);
  return 0;
}
