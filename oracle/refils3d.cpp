// refils3d.cpp -- runs the reference's ILS3D::Jacobi and ILS3D::BiCGSTAB
// (examples/SolverTest/ILS3D.h:478-529, 663-844, compiled from the
// reference's header) on the reference's BlockManager and
// Scalar3DUpdater<double>, with the Fortran loop bodies taken from the
// oracle (oracle/ils3d_shim.c) and a stand-in LocalScalar3D
// (oracle/ils3d/LocalScalar3D.h).  TEST INFRASTRUCTURE ONLY: the CPU tests
// compare its iteration counts, residuals and fields with the oracle's
// restatement of the same solvers, pinning their control flow to the
// reference's own code.  Built by oracle/Makefile into oracle/_ref/.
//
//   refils3d <in> <out>
//
// <in> (little endian): int32 rx, ry, rz, periodic_mask, n, vc, nb, mode
// (0 Jacobi, 1 BiCGSTAB), n_pre, max_iter; double omega, eps; uint64
// pedigree[nb]; then nine fields of nb packed bricks of (n+2vc)^3 doubles:
// Ap, Aw, Ae, As, An, Ab, At (boundary folded), b, x.
// <out>: int32 count; double residual; nb bricks of x after the solve.
// Blocks keep the pedigree list's order (BCMOctree(RootGrid*, pedigrees),
// Utils/src/BCMOctree.cpp:66-96).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "BCMOctree.h"
#include "BCMTools.h"
#include "Block.h"
#include "BlockFactory.h"
#include "BlockManager.h"
#include "BoundaryConditionSetterBase.h"
#include "BoundaryInfo.h"
#include "Partition.h"
#include "RootGrid.h"
#include "Scalar3D.h"
#include "Scalar3DUpdater.h"
#include "LocalScalar3D.h"
#include "ILS3D.h"

// No boundary condition objects: the outer faces are folded into the
// coefficient bricks by the caller.
class NoBoundary : public BoundaryConditionSetterBase {
 public:
  BoundaryInfo* operator()(const Node*, const BCMOctree*) { return new BoundaryInfo[NUM_FACE]; }
};

template <typename V>
static bool rd(FILE* fp, V* v, size_t n) { return fread(v, sizeof(V), n, fp) == n; }

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: refils3d <in> <out>\n");
    return 2;
  }
  FILE* fp = fopen(argv[1], "rb");
  if (!fp) return 3;
  int hdr[10];
  double om_eps[2];
  if (!rd(fp, hdr, 10) || !rd(fp, om_eps, 2)) return 3;
  const int rx = hdr[0], ry = hdr[1], rz = hdr[2], pmask = hdr[3], n = hdr[4], vc = hdr[5],
            nb = hdr[6], mode = hdr[7], n_pre = hdr[8], max_iter = hdr[9];
  std::vector<uint64_t> ped(nb);
  if (!rd(fp, ped.data(), nb)) return 3;
  const int n0 = n + 2 * vc;
  const size_t bsz = (size_t)n0 * n0 * n0;
  std::vector<double> in((size_t)9 * nb * bsz);
  if (!rd(fp, in.data(), in.size())) return 3;
  fclose(fp);

  RootGrid* root = new RootGrid(rx, ry, rz);
  if (pmask & 1) root->setPeriodicX();
  if (pmask & 2) root->setPeriodicY();
  if (pmask & 4) root->setPeriodicZ();
  std::vector<Pedigree> peds(nb);
  for (int b = 0; b < nb; b++) peds[b].deserialize(&ped[b]);
  BCMOctree* tree = new BCMOctree(root, peds);
  if (tree->getNumLeafNode() != nb) return 4;
  std::vector<Node*>& leaves = tree->getLeafNodeArray();
  Partition* part = new Partition(1, nb);
  NoBoundary* bcs = new NoBoundary;
  const Vec3i size(n, n, n);  // BlockFactory keeps a reference to it
  BlockFactory factory(tree, part, bcs, size);
  BlockManager& bm = BlockManager::getInstance();
  for (int b = 0; b < nb; b++) bm.registerBlock(factory.makeBlock(leaves[b]));
  bm.endRegisterBlock();

  LocalScalar3D<double> Ap(bm, vc), Aw(bm, vc), Ae(bm, vc), As(bm, vc), An(bm, vc), Ab(bm, vc),
      At(bm, vc), b(bm, vc), x(bm, vc);
  LocalScalar3D<double>* f9[9] = {&Ap, &Aw, &Ae, &As, &An, &Ab, &At, &b, &x};
  for (int q = 0; q < 9; q++)
    for (int k = 0; k < nb; k++) {
      double* d = f9[q]->GetBlockData(bm.getBlock(k));
      const double* s = &in[((size_t)q * nb + k) * bsz];
      for (size_t e = 0; e < bsz; e++) d[e] = s[e];
    }
  LocalScalar3D<double> r(bm, vc), r0(bm, vc), p(bm, vc), p_(bm, vc), q_(bm, vc), s(bm, vc),
      s_(bm, vc), t_(bm, vc), x0(bm, vc);
  ILS3D solver;
  int count = 0;
  double residual = 0.0;
  if (mode == 0) {
    solver.Jacobi(bm, &x, &Ap, &Aw, &Ae, &As, &An, &Ab, &At, &b, &x0, om_eps[0], max_iter,
                  om_eps[1], count, residual);
  } else {
    solver.BiCGSTAB(bm, &x, &Ap, &Aw, &Ae, &As, &An, &Ab, &At, &b, &r, &r0, &p, &p_, &q_, &s,
                    &s_, &t_, &x0, om_eps[0], n_pre, max_iter, om_eps[1], count, residual);
  }
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 6;
  fwrite(&count, 4, 1, out);
  fwrite(&residual, 8, 1, out);
  for (int k = 0; k < nb; k++) fwrite(x.GetBlockData(bm.getBlock(k)), 8, bsz, out);
  fclose(out);
  return 0;
}
