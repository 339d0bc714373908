/*
 * BlockManager.h -- source-compatible BlockManager for the GB300 drop-in.
 *
 * Same class names and members as BCMTools 1.0.5's VCUpdateMethod and
 * BlockManager (include/BlockManager.h:40-866, src/BlockManager.cpp), so an
 * application recompiles against it unchanged: put include/bcmtools (this
 * directory) ahead of the reference's include/ on the include path, keep the
 * reference's other headers and its Utils library for the mesh, and link
 * libbcmg.so instead of the reference's BlockManager.cpp and CommBuffer.cpp.
 *
 * What changes behind the interface:
 *  - endRegisterBlock (BlockManager.cpp:35-59) also hands the blocks'
 *    NeighborInfo tables to a libbcmg.so context on one GPU (the device of
 *    BCMG_DEVICE, default 0), which builds the device face table;
 *  - setDataClass<Scalar3D<T>, Scalar3DUpdater<T> >(vc) and the contiguous
 *    setDataClass<D,U,T> (BlockManager.h:226-283) give every block a brick of
 *    one libbcmg.so field in page-locked host memory mapped into the GPU's
 *    address space: host code reads and writes getData() as before;
 *  - beginUpdateVC / endUpdateVC and all their per-axis and per-level-
 *    difference variants (BlockManager.h:311-726) update every selected ghost
 *    face in one device launch with the reference's arithmetic (bit-exact in
 *    double, C2F within one ulp in float), complete when beginUpdateVC
 *    returns -- as the reference finishes its local copies there -- so host
 *    code may touch the field right after it; endUpdateVC has nothing left
 *    to wait for on one rank;
 *  - one process drives one GPU: every neighbour is local, there is no MPI
 *    exchange and no CommBuffer; a communicator of more than one rank is
 *    refused.
 * Data classes whose updater is not this directory's Scalar3DUpdater<T> are
 * refused at setDataClass (the reference's other updaters are per-face CPU
 * code); setDataClass<D>(vc) without an updater is the reference's.
 *
 * Errors print a message and exit, as the reference's Exit() does
 * (BCMTools.h:36-37).
 */
#ifndef BCMG_COMPAT_BLOCK_MANAGER_H
#define BCMG_COMPAT_BLOCK_MANAGER_H

#include "mpi.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <vector>

#include "BCMTools.h"
#include "BlockBase.h"
#include "Scalar3D.h"
#include "bcmg.h"

class VCUpdateMethod {
 public:
  enum Type {
    AtOnce,
    SeparateXYZ,
    SeparateXYZ_SeparateLevelDiff,
  };
};

namespace bcmg_compat {

// Element type code of the data classes the device updates.
template <typename D>
struct DeviceData {
  enum { ok = 0, code = -1 };
};
template <>
struct DeviceData<Scalar3D<float> > {
  enum { ok = 1, code = BCMG_F32 };
  typedef float value_type;
};
template <>
struct DeviceData<Scalar3D<double> > {
  enum { ok = 1, code = BCMG_F64 };
  typedef double value_type;
};

// True for updaters that declare bcmg_device_updater (Scalar3DUpdater<T>).
template <typename U>
struct IsDeviceUpdater {
  typedef char yes[1];
  typedef char no[2];
  template <typename V>
  static yes& test(int (*)[V::bcmg_device_updater]);
  template <typename V>
  static no& test(...);
  enum { value = sizeof(test<U>(0)) == sizeof(yes) };
};

}  // namespace bcmg_compat

class BlockManager {
  enum LevelDiff { LD_M1, LD_0, LD_P1 };
  typedef std::vector<BlockBase*> BlockList;

  int startID;
  int numBlock;
  MPI::Intracomm comm;
  BlockList blockList;
  Vec3i size;
  bcmg_ctx ctx;
  std::map<int, int> deviceField;  // data class id -> libbcmg.so field

  BlockManager() : startID(0), numBlock(0), comm(MPI::COMM_WORLD), size(0), ctx(0) {}
  BlockManager(const BlockManager&);
  BlockManager& operator=(const BlockManager&);

  void check(int rc, const char* what) const {
    if (rc != BCMG_SUCCESS) {
      std::cout << "*** error: " << what << ": " << (ctx ? bcmg_last_error(ctx) : "no context")
                << " (status " << rc << ")" << std::endl;
      Exit(EX_FAILURE);
    }
  }

  int fieldOf(int dataClassID) const {
    std::map<int, int>::const_iterator it = deviceField.find(dataClassID);
    if (it == deviceField.end()) {
      std::cout << "*** error: data class " << dataClassID
                << " has no device updater (setDataClass<Scalar3D<T>, Scalar3DUpdater<T> >)"
                << std::endl;
      Exit(EX_FAILURE);
    }
    return it->second;
  }

  // One device launch over the selected faces, waited for.  axisMask bit a:
  // faces normal to axis a; ldMask bit (d+1): level difference d.
  void update(int dataClassID, int axisMask, int ldMask) {
    const int f = fieldOf(dataClassID);
    check(bcmg_vc_begin(ctx, f, axisMask, ldMask, 0), "beginUpdateVC");
    check(bcmg_vc_end(ctx, f), "beginUpdateVC");
  }

  template <typename D, typename U>
  int setDeviceDataClass(int vc, const char* what) {
    typedef typename bcmg_compat::DeviceData<D>::value_type T;
    if (!ctx) {
      std::cout << "*** error: " << what << " before endRegisterBlock" << std::endl;
      Exit(EX_FAILURE);
    }
    int field = -1;
    check(bcmg_field_create_host(ctx, bcmg_compat::DeviceData<D>::code, vc, &field), what);
    void* base = 0;
    int64_t stride = 0;
    check(bcmg_field_layout(ctx, field, &base, &stride, 0), what);
    int id = -1;
    for (int b = 0; b < numBlock; b++) {
      BlockBase* block = blockList[b];
      D* dataClass = new D(block->getSize(), vc, static_cast<T*>(base) + (size_t)b * stride);
      U* updater = new U(block->getNeighborInfo());
      dataClass->setUpdater(updater);
      int id0 = block->setDataClass(dataClass);
      if (b == 0) {
        id = id0;
      } else if (id != id0) {
        std::cout << "error: DataClass register inconsistency" << std::endl;
        Exit(EX_FAILURE);
      }
    }
    deviceField[id] = field;
    return id;
  }

  template <typename D, typename U, bool device>
  struct Dispatch;

  template <typename D, typename U>
  struct Dispatch<D, U, true> {
    static int run(BlockManager* m, int vc, const char* what) {
      return m->template setDeviceDataClass<D, U>(vc, what);
    }
  };

  template <typename D, typename U>
  struct Dispatch<D, U, false> {
    static int run(BlockManager*, int, const char*) {
      std::cout << "*** error: this BlockManager updates ghost cells on the GPU; the updater of "
                   "setDataClass<D, U> must be Scalar3DUpdater<float> or Scalar3DUpdater<double> "
                   "over Scalar3D of the same type"
                << std::endl;
      Exit(EX_FAILURE);
      return -1;
    }
  };

  void layoutInfo(std::ostream& os) const {
    int levelMin = INT_MAX, levelMax = 0;
    for (int b = 0; b < numBlock; b++) {
      levelMin = std::min(levelMin, blockList[b]->getLevel());
      levelMax = std::max(levelMax, blockList[b]->getLevel());
    }
    os << "Block Layout Information" << std::endl;
    os << "  Min level: " << levelMin << std::endl;
    os << "  Max level: " << levelMax << std::endl;
    std::vector<int> perLevel(levelMax - levelMin + 1, 0);
    for (int b = 0; b < numBlock; b++) perLevel[blockList[b]->getLevel() - levelMin]++;
    os << "  Number of blocks" << std::endl;
    for (int l = levelMin; l <= levelMax; l++)
      os << "    L=" << l << ": " << perLevel[l - levelMin] << std::endl;
    os << "    total: " << numBlock << std::endl;
    os << "  Number of total blocks / node" << std::endl;
    os << "    ave: " << (REAL_TYPE)numBlock << std::endl;
    os << "    min: " << numBlock << std::endl;
    os << "    max: " << numBlock << std::endl;
    os << "     sd: " << (REAL_TYPE)0 << std::endl;
    // faces with a neighbour: one per face at level difference 0 and -1,
    // one per existing subface at +1; all intra-node on one rank
    int intra[3] = {0, 0, 0};
    for (int b = 0; b < numBlock; b++) {
      const NeighborInfo* ni = blockList[b]->getNeighborInfo();
      for (int f = 0; f < NUM_FACE; f++) {
        const int d = ni[f].getLevelDifference();
        const int nsub = d == 1 ? NUM_SUBFACE : 1;
        for (int s = 0; s < nsub; s++)
          if (ni[f].getID(Subface(s)) >= 0 && d >= -1 && d <= 1) intra[d + 1]++;
      }
    }
    os << "  Number of faces" << std::endl;
    os << "    intra-node " << std::endl;
    os << "        dLevel=-1: " << intra[LD_M1] << std::endl;
    os << "        dLevel= 0: " << intra[LD_0] << std::endl;
    os << "        dLevel=+1: " << intra[LD_P1] << std::endl;
    os << "            total: " << intra[LD_M1] + intra[LD_0] + intra[LD_P1] << std::endl;
    os << "    inter-node " << std::endl;
    os << "        dLevel=-1: " << 0 << std::endl;
    os << "        dLevel= 0: " << 0 << std::endl;
    os << "        dLevel=+1: " << 0 << std::endl;
    os << "            total: " << 0 << std::endl;
    os << "  Number of total inter-node faces / node" << std::endl;
    os << "    ave: " << (REAL_TYPE)0 << std::endl;
    os << "    min: " << 0 << std::endl;
    os << "    max: " << 0 << std::endl;
    os << "     sd: " << (REAL_TYPE)0 << std::endl;
  }

 public:
  static BlockManager& getInstance() {
    static BlockManager instance;
    return instance;
  }

  void setCommunicator(const MPI::Intracomm& c) { comm = c; }

  const MPI::Intracomm& getCommunicator() { return comm; }

  void registerBlock(BlockBase* block) {
    blockList.push_back(block);
    numBlock++;
  }

  /// BlockManager::endRegisterBlock (BlockManager.cpp:35-59) plus the device
  /// context and face table of the registered mesh.
  void endRegisterBlock() {
    if (numBlock == 0) {
      std::cout << "***error: number of blocks must be > 0" << std::endl;
      Exit(EX_FAILURE);
    }
    for (int i = 0; i < numBlock; i++) {
      if (i == 0) {
        size = blockList[i]->getSize();
      } else if (size != blockList[i]->getSize()) {
        std::cout << "***error: block size inconsistent" << std::endl;
        Exit(EX_FAILURE);
      }
    }
    if (comm.Get_size() != 1) {
      std::cout << "*** error: the GPU BlockManager runs one process per GPU with every "
                   "neighbour local; got " << comm.Get_size() << " ranks" << std::endl;
      Exit(EX_FAILURE);
    }
    startID = 0;
    std::vector<int> ld(numBlock * NUM_FACE), id(numBlock * NUM_FACE * NUM_SUBFACE),
        sf(numBlock * NUM_FACE);
    for (int b = 0; b < numBlock; b++) {
      const NeighborInfo* ni = blockList[b]->getNeighborInfo();
      for (int f = 0; f < NUM_FACE; f++) {
        const int k = b * NUM_FACE + f;
        ld[k] = ni[f].getLevelDifference();
        for (int s = 0; s < NUM_SUBFACE; s++) id[k * NUM_SUBFACE + s] = ni[f].getID(Subface(s));
        sf[k] = ni[f].getLevelDifference() == -1 ? (int)ni[f].getNeighborSubface() : 0;
      }
    }
    if (!ctx) {
      const char* dev = std::getenv("BCMG_DEVICE");
      check(bcmg_ctx_create(&ctx, dev ? std::atoi(dev) : 0), "endRegisterBlock");
    }
    check(bcmg_register_blocks(ctx, numBlock, size[0], size[1], size[2], &ld[0], &id[0], &sf[0]),
          "endRegisterBlock");
  }

  const Vec3i& getSize() const { return size; }

  int getStartID() const { return startID; }

  int getNumBlock() const { return numBlock; }

  BlockBase* getBlock(int localID) {
    if (localID < 0 || localID >= numBlock) {
      std::cout << "***error: illegal local block ID" << std::endl;
      Exit(EX_FAILURE);
    }
    return blockList[localID];
  }

  /// BlockManager::printBlockLayoutInfo (BlockManager.cpp:118-288), one rank.
  void printBlockLayoutInfo() { layoutInfo(std::cout); }

  void printBlockLayoutInfo(const char* filename) {
    std::ofstream ofs(filename, std::ios::out);
    layoutInfo(ofs);
  }

  /// setDataClass<D>(vc): a data class without updater, as the reference's.
  template <typename D>
  int setDataClass(int vc) {
    int id = -1;
    for (int b = 0; b < numBlock; b++) {
      int id0 = blockList[b]->setDataClass(new D(blockList[b]->getSize(), vc));
      if (b == 0) {
        id = id0;
      } else if (id != id0) {
        std::cout << "error: DataClass register inconsistency" << std::endl;
        Exit(EX_FAILURE);
      }
    }
    return id;
  }

  /// setDataClass<Scalar3D<T>, Scalar3DUpdater<T> >(vc): bricks of one
  /// host-visible device field, ghost updates on the GPU.
  template <typename D, typename U>
  int setDataClass(int vc) {
    return Dispatch < D, U,
           bcmg_compat::DeviceData<D>::ok && bcmg_compat::IsDeviceUpdater<U>::value >
               ::run(this, vc, "setDataClass");
  }

  /// The contiguous form: the same, since the field is one allocation.
  template <typename D, typename U, typename T>
  int setDataClass(int vc) {
    return setDataClass<D, U>(vc);
  }

  void prepareForVCUpdate(int dataClassID, int tag, VCUpdateMethod::Type method) {
    check(bcmg_prepare_vc(ctx, fieldOf(dataClassID), tag, (int)method), "prepareForVCUpdate");
  }

  void prepareForVCUpdate(int dataClassID, int tag, bool separate = false) {
    prepareForVCUpdate(dataClassID, tag,
                       separate ? VCUpdateMethod::SeparateXYZ : VCUpdateMethod::AtOnce);
  }

  void updateVC(int dataClassID) { update(dataClassID, 7, 7); }
  void updateVC(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 7); }
  void updateVC_Flat(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 2); }
  void updateVC_F2C(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 4); }
  void updateVC_C2F(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 1); }
  void updateVC_X(int id) { updateVC(id, 0); }
  void updateVC_Y(int id) { updateVC(id, 1); }
  void updateVC_Z(int id) { updateVC(id, 2); }
  void updateVC_X_Flat(int id) { updateVC_Flat(id, 0); }
  void updateVC_Y_Flat(int id) { updateVC_Flat(id, 1); }
  void updateVC_Z_Flat(int id) { updateVC_Flat(id, 2); }
  void updateVC_X_F2C(int id) { updateVC_F2C(id, 0); }
  void updateVC_Y_F2C(int id) { updateVC_F2C(id, 1); }
  void updateVC_Z_F2C(int id) { updateVC_F2C(id, 2); }
  void updateVC_X_C2F(int id) { updateVC_C2F(id, 0); }
  void updateVC_Y_C2F(int id) { updateVC_C2F(id, 1); }
  void updateVC_Z_C2F(int id) { updateVC_C2F(id, 2); }

  void beginUpdateVC(int dataClassID) { update(dataClassID, 7, 7); }
  void beginUpdateVC(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 7); }
  void beginUpdateVC_Flat(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 2); }
  void beginUpdateVC_F2C(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 4); }
  void beginUpdateVC_C2F(int dataClassID, int xyz) { update(dataClassID, 1 << xyz, 1); }
  void beginUpdateVC_X(int id) { beginUpdateVC(id, 0); }
  void beginUpdateVC_Y(int id) { beginUpdateVC(id, 1); }
  void beginUpdateVC_Z(int id) { beginUpdateVC(id, 2); }
  void beginUpdateVC_X_Flat(int id) { beginUpdateVC_Flat(id, 0); }
  void beginUpdateVC_Y_Flat(int id) { beginUpdateVC_Flat(id, 1); }
  void beginUpdateVC_Z_Flat(int id) { beginUpdateVC_Flat(id, 2); }
  void beginUpdateVC_X_F2C(int id) { beginUpdateVC_F2C(id, 0); }
  void beginUpdateVC_Y_F2C(int id) { beginUpdateVC_F2C(id, 1); }
  void beginUpdateVC_Z_F2C(int id) { beginUpdateVC_F2C(id, 2); }
  void beginUpdateVC_X_C2F(int id) { beginUpdateVC_C2F(id, 0); }
  void beginUpdateVC_Y_C2F(int id) { beginUpdateVC_C2F(id, 1); }
  void beginUpdateVC_Z_C2F(int id) { beginUpdateVC_C2F(id, 2); }

  // the device work is complete when beginUpdateVC* returns
  void endUpdateVC(int dataClassID) { fieldOf(dataClassID); }
  void endUpdateVC(int dataClassID, int) { fieldOf(dataClassID); }
  void endUpdateVC_Flat(int dataClassID, int) { fieldOf(dataClassID); }
  void endUpdateVC_F2C(int dataClassID, int) { fieldOf(dataClassID); }
  void endUpdateVC_C2F(int dataClassID, int) { fieldOf(dataClassID); }
  void endUpdateVC_X(int id) { endUpdateVC(id, 0); }
  void endUpdateVC_Y(int id) { endUpdateVC(id, 1); }
  void endUpdateVC_Z(int id) { endUpdateVC(id, 2); }
  void endUpdateVC_X_Flat(int id) { endUpdateVC_Flat(id, 0); }
  void endUpdateVC_Y_Flat(int id) { endUpdateVC_Flat(id, 1); }
  void endUpdateVC_Z_Flat(int id) { endUpdateVC_Flat(id, 2); }
  void endUpdateVC_X_F2C(int id) { endUpdateVC_F2C(id, 0); }
  void endUpdateVC_Y_F2C(int id) { endUpdateVC_F2C(id, 1); }
  void endUpdateVC_Z_F2C(int id) { endUpdateVC_F2C(id, 2); }
  void endUpdateVC_X_C2F(int id) { endUpdateVC_C2F(id, 0); }
  void endUpdateVC_Y_C2F(int id) { endUpdateVC_C2F(id, 1); }
  void endUpdateVC_Z_C2F(int id) { endUpdateVC_C2F(id, 2); }

  /// The libbcmg.so context and the field behind a device data class, for
  /// code that moves its own sweeps to the library's kernels too.
  bcmg_ctx getDeviceContext() const { return ctx; }
  int getDeviceField(int dataClassID) const { return fieldOf(dataClassID); }
};

#endif  // BCMG_COMPAT_BLOCK_MANAGER_H
