/*
 * LocalScalar3D.h -- project-written stand-in for SolverTest's
 * LocalScalar3D<T> (examples/SolverTest/LocalScalar3D.h), with only what
 * ILS3D.h calls: GetVC, GetBlockData, ImposeBoundaryCondition,
 * UpdateVirtualCells and LSSwap.  TEST INFRASTRUCTURE ONLY: it lets the
 * reference's ILS3D.h compile here, around the reference's own BlockManager
 * and Scalar3DUpdater<T>, so that its solvers' control flow can be compared
 * with the oracle's restatement (oracle/refils3d.cpp).
 *
 * The real class also selects an updater type and applies per-face boundary
 * functions (bcx.f90).  The systems this stand-in serves have their outer
 * faces folded into the coefficient bricks (bca.f90: the neighbour
 * coefficient there is zero), so the outer ghost values never enter a result
 * and ImposeBoundaryCondition is the reference's ghost update alone
 * (LocalScalar3D.h:228-258 without its boundary-function part).
 */
#ifndef BCMG_ILS3D_LOCAL_SCALAR3D_H
#define BCMG_ILS3D_LOCAL_SCALAR3D_H

#include <algorithm>

#include "BlockManager.h"
#include "Scalar3D.h"
#include "Scalar3DUpdater.h"

template <typename T>
class LocalScalar3D {
  int vc;
  int id;

 public:
  LocalScalar3D(BlockManager& bm, int vc) : vc(vc) {
    id = bm.setDataClass<Scalar3D<T>, Scalar3DUpdater<T> >(vc);
    bm.prepareForVCUpdate(id, 100, false);
  }
  int GetVC() const { return vc; }
  int GetID() const { return id; }
  T* GetBlockData(BlockBase* block) const {
    return dynamic_cast<Scalar3D<T>*>(block->getDataClass(id))->getData();
  }
  void ImposeBoundaryCondition(BlockManager& bm) { bm.updateVC(id); }
  // UpdateVirtualCells (LocalScalar3D.h:199-230), the AtOnce method
  void UpdateVirtualCells(BlockManager& bm) { bm.updateVC(id); }
  // LSSwap (LocalScalar3D.h:132-136): the two objects exchange their data
  friend void LSSwap(LocalScalar3D& a, LocalScalar3D& b) { std::swap(a.id, b.id); }
};

#endif
