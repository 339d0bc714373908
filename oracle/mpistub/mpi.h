/*
 * Single-rank stand-in for the MPI C++ bindings, written for this project.
 *
 * Test infrastructure only: it lets the reference library's own C++ sources
 * (BlockManager, CommBuffer, BCMOctree, the sor1 example) compile and run as
 * one process, so their results can serve as the oracle for the GPU path.
 * Collectives degenerate to copies; point-to-point calls abort, because with
 * one rank every neighbouring block is local and the reference never reaches
 * its send/receive code (BlockManager.cpp:487-506 puts every face in the
 * local list when neighbour rank == my rank).
 */
#ifndef BCMG_ORACLE_MPISTUB_H
#define BCMG_ORACLE_MPISTUB_H

#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_IN_PLACE ((void*)1)
#define MPI_SUCCESS 0

namespace MPI {

typedef int Datatype;
typedef int Op;

static const Datatype CHAR = 1, INT = 4, DOUBLE = 8, BYTE = 101, FLOAT = 104;
static const Op SUM = 0, MIN = 1, MAX = 2;
static const int PROC_NULL = -2;
static void* const IN_PLACE = MPI_IN_PLACE;

inline size_t type_size(Datatype t) {
  switch (t) {
    case CHAR: case BYTE: return 1;
    case INT: case FLOAT: return 4;
    case DOUBLE: return 8;
    default: return 1;
  }
}

inline void stub_fail(const char* what) {
  std::fprintf(stderr, "mpi stub: %s is unreachable on one rank\n", what);
  std::abort();
}

class Status {
 public:
  int Get_source() const { return 0; }
};

class Request {
 public:
  static void Waitall(int n, Request*, Status*) {
    if (n != 0) stub_fail("Waitall with pending requests");
  }
};

class Comm {
 public:
  virtual ~Comm() {}
  int Get_rank() const { return 0; }
  int Get_size() const { return 1; }
  void Barrier() const {}
  void Abort(int code) const { std::exit(code); }
  void Send(const void*, int, Datatype, int, int) const { stub_fail("Send"); }
  void Recv(void*, int, Datatype, int, int) const { stub_fail("Recv"); }
  void Recv(void*, int, Datatype, int, int, Status&) const { stub_fail("Recv"); }
  Request Isend(const void*, int, Datatype, int, int) const {
    stub_fail("Isend");
    return Request();
  }
  Request Irecv(void*, int, Datatype, int, int) const {
    stub_fail("Irecv");
    return Request();
  }
  void Bcast(void*, int, Datatype, int) const {}
  void Reduce(const void* s, void* r, int n, Datatype t, Op, int) const {
    if (s != IN_PLACE && s != r) std::memcpy(r, s, n * type_size(t));
  }
  void Allreduce(const void* s, void* r, int n, Datatype t, Op) const {
    if (s != IN_PLACE && s != r) std::memcpy(r, s, n * type_size(t));
  }
  void Scan(const void* s, void* r, int n, Datatype t, Op) const {
    if (s != IN_PLACE && s != r) std::memcpy(r, s, n * type_size(t));
  }
  void Gather(const void* s, int n, Datatype t, void* r, int, Datatype, int) const {
    if (s != IN_PLACE && s != r) std::memcpy(r, s, n * type_size(t));
  }
};

class Intracomm : public Comm {};

extern Intracomm COMM_WORLD;

inline void Init(int&, char**&) {}
inline void Init() {}
inline void Finalize() {}

}  // namespace MPI

#endif
