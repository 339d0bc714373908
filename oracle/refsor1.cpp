// refsor1.cpp -- runs the reference's examples/sor1 Solver (its own
// Solver.cpp, compiled from the reference sources) on a config file and
// dumps every block's pedigree and padded field after Solver::run.
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/.
//
//   refsor1 <config> <out>
// Output: int32 nb, n, vc; per block uint64 pedigree, int32 level,
// double origin[3], double cellSize[3], int32 bcType[6] (BoundaryInfo::Type),
// int32 bcId[6], int32 {ld,id0..id3,sf}[6]; then nb bricks of double.
// The block setup mirrors sor1/main.cpp:66-145 (the reference's own flow).
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
  if (conf.type == 'x') { rootGrid->setPeriodicY(); rootGrid->setPeriodicZ(); }
  if (conf.type == 'y') { rootGrid->setPeriodicZ(); rootGrid->setPeriodicX(); }
  if (conf.type == 'z') { rootGrid->setPeriodicX(); rootGrid->setPeriodicY(); }
  Divider* divider = (conf.treeType == "flat")
      ? (Divider*)new FlatDivider(rootGrid, conf.maxLevel)
      : (Divider*)new SimpleDivider(rootGrid, conf.minLevel, conf.maxLevel);
  BCMOctree* tree = new BCMOctree(rootGrid, divider, BCMOctree::Z);
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
  // Two entries: the reference's main writes boundaryValue[1] past a
  // one-element vector (sor1/main.cpp:141-143); here the vector is sized 2.
  std::vector<double> boundaryValue(2);
  boundaryValue[0] = conf.b0;
  boundaryValue[1] = conf.b1;
  Solver solver(conf, boundaryValue);
  solver.initialize();
  solver.run();
  solver.checkResult(conf.type, false);

  FILE* fp = fopen(argv[2], "wb");
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
  int n0 = conf.size + 2 * conf.vc;
  for (int b = 0; b < nb; b++) {
    Scalar3D<double>* f = dynamic_cast<Scalar3D<double>*>(bm.getBlock(b)->getDataClass(0));
    fwrite(f->getData(), 8, (size_t)n0 * n0 * n0, fp);
  }
  fclose(fp);
  return 0;
}
