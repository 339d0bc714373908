/*
 * Scalar3D.h -- source-compatible Scalar3D<T> for the GB300 drop-in.
 *
 * Same class name, constructors and members as BCMTools 1.0.5's Scalar3D<T>
 * (include/Scalar3D.h:37-277): a padded brick of (nx+2vc)(ny+2vc)(nz+2vc)
 * values, x fastest, cell (i,j,k) at i + nx0 j + nx0 ny0 k + (1+nx0+nx0 ny0) vc,
 * with the box copies the reference's updater used.  The differences:
 *
 *  - the three-argument constructor over caller storage does not own that
 *    storage (the reference's destructor deletes it, Scalar3D.h:88-90, which
 *    breaks its own contiguous setDataClass<D,U,T>); the drop-in BlockManager
 *    hands every block a brick of one field of libbcmg.so in page-locked host
 *    memory that the GPU reaches directly, so host code keeps reading and
 *    writing getData() as before while the ghost update runs on the device;
 *  - the box copies are plain loops (no OpenMP inside a block).
 *
 * Put include/bcmtools ahead of the reference's include/ on the include path:
 * the other reference headers (BCMTools.h, Vec3.h, Index3D.h, DataClass.h,
 * VCUpdater.h, BlockBase.h, NeighborInfo.h) are used as they are.
 */
#ifndef BCMG_COMPAT_SCALAR3D_H
#define BCMG_COMPAT_SCALAR3D_H

#include "DataClass.h"
#include "Index3D.h"
#include "VCUpdater.h"

template <typename T>
class Scalar3D : public UpdatableDataClass {
  int nx0, ny0, nz0;
  int c_0, c_j, c_k;
  T* data;
  bool owner;  // storage from new[] in the two-argument constructor
  Index3DS index;
  int vc0;

  void init(const ::Vec3i& size, int vc) {
    nx0 = size[0] + 2 * vc;
    ny0 = size[1] + 2 * vc;
    nz0 = size[2] + 2 * vc;
    vc0 = vc;
    c_j = nx0;
    c_k = nx0 * ny0;
    c_0 = (1 + nx0 + nx0 * ny0) * vc;
  }

  Scalar3D(const Scalar3D&);
  Scalar3D& operator=(const Scalar3D&);

 public:
  /// Brick of its own (host memory), as Scalar3D(size, vc) of the reference.
  Scalar3D(const ::Vec3i& size, int vc)
      : UpdatableDataClass(size, vc), owner(true), index(size, vc) {
    init(size, vc);
    data = new T[(size_t)nx0 * ny0 * nz0]();
  }

  /// Brick in caller storage (contiguous fields); the storage stays the caller's.
  Scalar3D(const ::Vec3i& size, int vc, T* data0)
      : UpdatableDataClass(size, vc), data(data0), owner(false), index(size, vc) {
    init(size, vc);
  }

  ~Scalar3D() {
    if (owner) delete[] data;
  }

  T* getData() const { return data; }

  int getVCsize() { return vc0; }

  Index3DS getIndex() const { return index; }

  T& operator()(int i, int j, int k) { return data[i + c_j * j + c_k * k + c_0]; }

  const T& operator()(int i, int j, int k) const { return data[i + c_j * j + c_k * k + c_0]; }

  void copyToBuffer(int i0, int j0, int k0, int nx, int ny, int nz, T* buffer) const {
    size_t q = 0;
    for (int k = k0; k < k0 + nz; ++k)
      for (int j = j0; j < j0 + ny; ++j)
        for (int i = i0; i < i0 + nx; ++i) buffer[q++] = data[index(i, j, k)];
  }

  void copyFromBuffer(int i0, int j0, int k0, int nx, int ny, int nz, const T* buffer) {
    size_t q = 0;
    for (int k = k0; k < k0 + nz; ++k)
      for (int j = j0; j < j0 + ny; ++j)
        for (int i = i0; i < i0 + nx; ++i) data[index(i, j, k)] = buffer[q++];
  }

  void copyFromDataClass(int i0, int j0, int k0, int i1, int j1, int k1, int nx, int ny, int nz,
                         const DataClass* dataClass) {
    const Scalar3D<T>* s = dynamic_cast<const Scalar3D<T>*>(dataClass);
    const T* sData = s->getData();
    Index3DS sIndex = s->getIndex();
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          data[index(i0 + i, j0 + j, k0 + k)] = sData[sIndex(i1 + i, j1 + j, k1 + k)];
  }
};

#endif  // BCMG_COMPAT_SCALAR3D_H
