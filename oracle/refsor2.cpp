// refsor2.cpp -- runs the reference's examples/sor2 Solver (its own
// Solver.cpp, compiled from the reference sources) on a config file and
// dumps every block's tables, the final field and the source term.
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/.
//
//   refsor2 <config> <out>
// Output: the block records of refsor1 (int32 nb, n, vc; per block uint64
// pedigree, int32 level, double origin[3], double cellSize[3], int32
// bcType[6], int32 bcId[6], int32 {ld,id0..id3,sf}[6]); then nb padded bricks
// of double (the field after Solver::run); then per block 3n doubles, the
// factors sin(a x_i), sin(a y_j), sin(a z_k) (a = 2 pi, cell centres) of
// sor2's source s = ((-3a^2 sx) sy) sz (Solver::setSource,
// examples/sor2/Solver.cpp:383-405), evaluated here with the same operations,
// compiler and libm, so that the product rebuilds the source bit for bit.
// The block setup follows sor2/main.cpp:63-138 (the reference's own flow).
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>
#include "BCMTools.h"
#include "Config.h"
#include "RootGrid.h"
#include "BCMOctree.h"
#include "SimpleDivider.h"
#include "Partition.h"
#include "BoundaryConditionSetter.h"
#include "BlockFactory.h"
#include "Block.h"
#include "BlockManager.h"
#include "Solver.h"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  Config conf;
  conf.load(argv[1]);
  RootGrid* rootGrid = new RootGrid(1, 1, 1);
  Divider* divider = (conf.treeType == "flat")
      ? (Divider*)new FlatDivider(rootGrid, conf.maxLevel)
      : (Divider*)new SimpleDivider(rootGrid, conf.minLevel, conf.maxLevel);
  BCMOctree::Ordering ordering = conf.ordering == "Hilbert" ? BCMOctree::HILBERT
                                 : conf.ordering == "random" ? BCMOctree::RANDOM
                                                             : BCMOctree::Z;
  BCMOctree* tree = new BCMOctree(rootGrid, divider, ordering);
  int nl = tree->getNumLeafNode();
  std::vector<Node*>& leaves = tree->getLeafNodeArray();
  Partition* partition = new Partition(1, nl);
  Vec3i size(conf.size, conf.size, conf.size);
  BoundaryConditionSetter* bcs = new BoundaryConditionSetter(&conf);
  BlockFactory* factory = new BlockFactory(tree, partition, bcs, size);
  BlockManager& bm = BlockManager::getInstance();
  std::vector<uint64_t> peds;
  for (int id = 0; id < nl; id++) {
    Block* block = factory->makeBlock(leaves[id]);
    bm.registerBlock(block);
    uint64_t p;
    leaves[id]->getPedigree().serialize(&p);
    peds.push_back(p);
  }
  bm.endRegisterBlock();
  std::vector<double> boundaryValue(1);
  boundaryValue[0] = 0.0;
  Solver solver(conf, boundaryValue);
  solver.initialize();
  solver.run();

  FILE* fp = fopen(argv[2], "wb");
  if (!fp) return 3;
  int nb = bm.getNumBlock();
  int hdr[3] = {nb, conf.size, conf.vc};
  fwrite(hdr, 4, 3, fp);
  for (int b = 0; b < nb; b++) {
    Block* block = dynamic_cast<Block*>(bm.getBlock(b));
    fwrite(&peds[b], 8, 1, fp);
    int level = block->getLevel();
    fwrite(&level, 4, 1, fp);
    double o[3] = {block->getOrigin().x, block->getOrigin().y, block->getOrigin().z};
    double c[3] = {block->getCellSize().x, block->getCellSize().y, block->getCellSize().z};
    fwrite(o, 8, 3, fp);
    fwrite(c, 8, 3, fp);
    const BoundaryInfo* bi = block->getBoundaryInfo();
    int bt[6], bid[6];
    for (int f = 0; f < 6; f++) { bt[f] = bi[f].getType(); bid[f] = bi[f].getID(); }
    fwrite(bt, 4, 6, fp);
    fwrite(bid, 4, 6, fp);
    const NeighborInfo* ni = block->getNeighborInfo();
    for (int f = 0; f < 6; f++) {
      int rec[6];
      rec[0] = ni[f].getLevelDifference();
      for (int s = 0; s < 4; s++) rec[1 + s] = ni[f].getID(Subface(s));
      rec[5] = ni[f].getNeighborSubface();
      fwrite(rec, 4, 6, fp);
    }
  }
  const int n = conf.size, n0 = n + 2 * conf.vc;
  for (int b = 0; b < nb; b++) {
    Scalar3D<double>* f = dynamic_cast<Scalar3D<double>*>(bm.getBlock(b)->getDataClass(0));
    fwrite(f->getData(), 8, (size_t)n0 * n0 * n0, fp);
  }
  // the source factors per block: sin(a x_i), sin(a y_j), sin(a z_k)
  std::vector<double> fac(3 * (size_t)n);
  for (int b = 0; b < nb; b++) {
    const Vec3d& orig = bm.getBlock(b)->getOrigin();
    const Vec3d& delta = bm.getBlock(b)->getCellSize();
    const double a = 2 * M_PI;
    for (int i = 0; i < n; ++i) {
      fac[i] = sin(a * (orig[0] + (i + 0.5) * delta[0]));
      fac[n + i] = sin(a * (orig[1] + (i + 0.5) * delta[1]));
      fac[2 * n + i] = sin(a * (orig[2] + (i + 0.5) * delta[2]));
    }
    fwrite(fac.data(), 8, fac.size(), fp);
  }
  fclose(fp);
  return 0;
}
