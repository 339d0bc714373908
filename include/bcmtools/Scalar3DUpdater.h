/*
 * Scalar3DUpdater.h -- the GB300 drop-in's VC updater, under the reference's
 * class name Scalar3DUpdater<T> (include/Scalar3DUpdater.h:43-904).
 *
 * It implements the reference's VCUpdater plugin interface
 * (include/VCUpdater.h:38-275), so setDataClass<Scalar3D<T>,
 * Scalar3DUpdater<T> >(vc) compiles and binds it as before.  Its per-face
 * hooks do nothing: the drop-in BlockManager (BlockManager.h in this
 * directory) updates every ghost face of a data class with this updater in
 * one device launch of libbcmg.so (same-level copy, fine-to-coarse average,
 * coarse-to-fine trilinear interpolation, with the reference's arithmetic),
 * instead of calling copyFromNeighbor once per face.  The multi-rank buffer
 * hooks report empty buffers: one process drives one GPU, every neighbour
 * is local.
 */
#ifndef BCMG_COMPAT_SCALAR3D_UPDATER_H
#define BCMG_COMPAT_SCALAR3D_UPDATER_H

#include "BCMTools.h"
#include "Scalar3D.h"
#include "VCUpdater.h"

template <typename T>
class Scalar3DUpdater : public VCUpdater {
  Scalar3D<T>* dataClass;

 public:
  /// Marks the updaters whose data classes the drop-in BlockManager updates
  /// on the device.
  enum { bcmg_device_updater = 1 };

  Scalar3DUpdater(const NeighborInfo* neighborInfo, const MPI::Comm& comm = MPI::COMM_WORLD)
      : VCUpdater(neighborInfo, comm), dataClass(0) {}

  ~Scalar3DUpdater() {}

  void setDataClass(DataClass* dc) { dataClass = dynamic_cast<Scalar3D<T>*>(dc); }

  void setNeighbor(Face, Subface, DataClass*) {}

  void clearNeighbor(Face, Subface) {}

  PointerSetterBase* getSendBufferPointerSetter(Face, Subface) { return 0; }

  PointerSetterBase* getRecvBufferPointerSetter(Face, Subface) { return 0; }

 private:
  void copyFromNeighbor(Face) {}
  void copyFromNeighborF2C(Face, Subface) {}
  void copyFromNeighborC2F(Face, Subface) {}
  void copyToCommBuffer(Face) {}
  void copyToCommBufferF2C(Face, Subface) {}
  void copyToCommBufferC2F(Face, Subface) {}
  void copyFromCommBuffer(Face) {}
  void copyFromCommBufferF2C(Face, Subface) {}
  void copyFromCommBufferC2F(Face, Subface) {}
  size_t getSendBufferByteSize(Face) const { return 0; }
  size_t getSendBufferByteSizeF2C(Face, Subface) const { return 0; }
  size_t getSendBufferByteSizeC2F(Face, Subface) const { return 0; }
  size_t getRecvBufferByteSize(Face) const { return 0; }
  size_t getRecvBufferByteSizeF2C(Face, Subface) const { return 0; }
  size_t getRecvBufferByteSizeC2F(Face, Subface) const { return 0; }
};

#endif  // BCMG_COMPAT_SCALAR3D_UPDATER_H
