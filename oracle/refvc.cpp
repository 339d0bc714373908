// refvc.cpp -- drives the reference library's own BCMOctree, BlockManager and
// Scalar3DUpdater<T> to produce golden data.  TEST INFRASTRUCTURE ONLY: built
// by oracle/Makefile from the reference sources into oracle/_ref/, never
// shipped.  Only the reference's public API is called.
//
//   refvc tree <rx> <ry> <rz> <pmask>
//              flat|simple|sphere:cx,cy,cz,r[,margin]|cylinder:cx,cy,r[,margin] <minL> <maxL>
//              Z|H <n> <out>
//       octree built by the reference's dividers (SimpleDivider.h,
//       SphereDivider.h, CylinderDivider.h), leaves in
//       Z or Hilbert order (BCMOctree.cpp:23-41), with makeNeighborInfo
//       (BCMOctree.cpp:423-478) for every leaf.
//   refvc vc <rx> <ry> <rz> <pmask> <pedigree-file> <n> <vc> <seed> <out>
//       octree from a pedigree list (BCMOctree.cpp:66-96); field of
//       Scalar3D<T> filled with seeded values in every cell; one
//       BlockManager::updateVC (BlockManager.h:311-315) through
//       Scalar3DUpdater<T>; writes the field before and after.
//
// Output (little endian): int32 nb, n, vc, sizeof(T); per block: uint64
// pedigree, int32 level, double origin[3], double blockSize[3], then per face
// int32 {ld, id0, id1, id2, id3, neighbourSubface}; then (vc mode) the nb
// bricks before and after the update.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>

#include "BCMTools.h"
#include "BlockManager.h"
#include "Scalar3D.h"
#include "Scalar3DUpdater.h"
#include "SphereDivider.h"
#include "CylinderDivider.h"
#include "RootGrid.h"
#include "BCMOctree.h"
#include "SimpleDivider.h"
#include "Partition.h"
#include "BlockFactory.h"
#include "BoundaryConditionSetterBase.h"
#include "BoundaryInfo.h"

#ifdef _REAL_IS_DOUBLE_
typedef double T;
#else
typedef float T;
#endif

class AllInner : public BoundaryConditionSetterBase {
 public:
  BoundaryInfo* operator()(const Node*, const BCMOctree*) { return new BoundaryInfo[NUM_FACE]; }
};

static uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static RootGrid* make_root(int rx, int ry, int rz, int pmask) {
  RootGrid* g = new RootGrid(rx, ry, rz);
  if (pmask & 1) g->setPeriodicX();
  if (pmask & 2) g->setPeriodicY();
  if (pmask & 4) g->setPeriodicZ();
  return g;
}

static void write_blocks(FILE* fp, BCMOctree* tree, int n, int vc, std::vector<Block*>& blocks) {
  int nb = tree->getNumLeafNode();
  int hdr[4] = {nb, n, vc, (int)sizeof(T)};
  fwrite(hdr, sizeof(int), 4, fp);
  std::vector<Node*>& leaves = tree->getLeafNodeArray();
  Partition* part = new Partition(1, nb);
  AllInner* bcs = new AllInner;
  Vec3i size(n, n, n);
  BlockFactory factory(tree, part, bcs, size);
  for (int id = 0; id < nb; id++) {
    Node* node = leaves[id];
    Block* block = factory.makeBlock(node);
    blocks.push_back(block);
    uint64_t ped;
    node->getPedigree().serialize(&ped);
    int level = node->getLevel();
    double o[3] = {block->getOrigin().x, block->getOrigin().y, block->getOrigin().z};
    double bs[3] = {block->getBlockSize().x, block->getBlockSize().y, block->getBlockSize().z};
    fwrite(&ped, 8, 1, fp);
    fwrite(&level, 4, 1, fp);
    fwrite(o, 8, 3, fp);
    fwrite(bs, 8, 3, fp);
    const NeighborInfo* ni = block->getNeighborInfo();
    for (int f = 0; f < NUM_FACE; f++) {
      int rec[6];
      rec[0] = ni[f].getLevelDifference();
      for (int s = 0; s < NUM_SUBFACE; s++) rec[1 + s] = ni[f].getID(Subface(s));
      rec[5] = ni[f].getNeighborSubface();
      fwrite(rec, 4, 6, fp);
    }
  }
  delete part;
  delete bcs;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::string mode = argv[1];
  if (mode == "tree" && argc == 12) {
    RootGrid* root = make_root(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), atoi(argv[5]));
    std::string kind = argv[6];
    int minL = atoi(argv[7]), maxL = atoi(argv[8]);
    Divider* div;
    double sc[5] = {0, 0, 0, 0, 0};
    if (kind == "flat")
      div = new FlatDivider(root, maxL);
    else if (sscanf(kind.c_str(), "sphere:%lf,%lf,%lf,%lf,%lf", &sc[0], &sc[1], &sc[2], &sc[3],
                    &sc[4]) >= 4)
      div = new SphereDivider(root, minL, maxL, sc[0], sc[1], sc[2], sc[3], sc[4]);
    else if (sscanf(kind.c_str(), "cylinder:%lf,%lf,%lf,%lf", &sc[0], &sc[1], &sc[2],
                    &sc[4]) >= 3)
      div = new CylinderDivider(root, minL, maxL, sc[0], sc[1], sc[2], sc[4]);
    else
      div = new SimpleDivider(root, minL, maxL);
    BCMOctree::Ordering ord = (std::string(argv[9]) == "H") ? BCMOctree::HILBERT : BCMOctree::Z;
    BCMOctree* tree = new BCMOctree(root, div, ord);
    FILE* fp = fopen(argv[11], "wb");
    std::vector<Block*> blocks;
    write_blocks(fp, tree, atoi(argv[10]), 1, blocks);
    fclose(fp);
    return 0;
  }
  if (mode == "vc" && argc == 11) {
    RootGrid* root = make_root(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), atoi(argv[5]));
    FILE* pf = fopen(argv[6], "rb");
    if (!pf) return 3;
    std::vector<Pedigree> peds;
    uint64_t p;
    while (fread(&p, 8, 1, pf) == 1) {
      Pedigree ped;
      ped.deserialize(&p);
      peds.push_back(ped);
    }
    fclose(pf);
    int n = atoi(argv[7]), vc = atoi(argv[8]);
    uint64_t seed = strtoull(argv[9], 0, 10);
    BCMOctree* tree = new BCMOctree(root, peds);
    FILE* fp = fopen(argv[10], "wb");
    std::vector<Block*> blocks;
    write_blocks(fp, tree, n, vc, blocks);
    BlockManager& bm = BlockManager::getInstance();
    for (size_t i = 0; i < blocks.size(); i++) bm.registerBlock(blocks[i]);
    bm.endRegisterBlock();
    int id = bm.setDataClass<Scalar3D<T>, Scalar3DUpdater<T> >(vc);
    bm.prepareForVCUpdate(id, 100, false);
    int n0 = n + 2 * vc;
    size_t bsz = (size_t)n0 * n0 * n0;
    uint64_t st = seed;
    for (int b = 0; b < bm.getNumBlock(); b++) {
      Scalar3D<T>* s = dynamic_cast<Scalar3D<T>*>(bm.getBlock(b)->getDataClass(id));
      T* d = s->getData();
      for (size_t e = 0; e < bsz; e++)
        d[e] = (T)((double)(splitmix(st) >> 11) * (2.0 / 9007199254740992.0) - 1.0);
      fwrite(d, sizeof(T), bsz, fp);
    }
    bm.updateVC(id);
    for (int b = 0; b < bm.getNumBlock(); b++) {
      Scalar3D<T>* s = dynamic_cast<Scalar3D<T>*>(bm.getBlock(b)->getDataClass(id));
      fwrite(s->getData(), sizeof(T), bsz, fp);
    }
    fclose(fp);
    return 0;
  }
  fprintf(stderr, "usage: see header of refvc.cpp\n");
  return 2;
}
