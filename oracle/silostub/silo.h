/*
 * Stand-in for the Silo file library's header, written for this project.
 *
 * Test infrastructure only: the reference's sor2 example includes its Silo
 * writer for the result check, which the oracle driver never calls.  These
 * declarations let that source compile and link unchanged; every function
 * does nothing and reports failure (null file, -1), so a call would write
 * nothing.
 */
#ifndef BCMG_ORACLE_SILOSTUB_H
#define BCMG_ORACLE_SILOSTUB_H

struct DBfile;
struct DBoptlist;

enum {
  DB_CLOBBER = 0, DB_LOCAL = 0, DB_PDB = 2, DB_HDF5 = 7,
  DB_INT = 16, DB_FLOAT = 19, DB_DOUBLE = 20,
  DB_ZONECENT = 111, DB_COLLINEAR = 130, DB_QUAD_RECT = 130, DB_QUADVAR = 501,
  DBOPT_HI_OFFSET = 1, DBOPT_LO_OFFSET, DBOPT_MB_BLOCK_NS, DBOPT_MB_BLOCK_TYPE,
  DBOPT_MB_FILE_NS, DBOPT_XLABEL, DBOPT_YLABEL, DBOPT_ZLABEL
};

template <typename... A> inline DBfile* DBCreate(A...) { return nullptr; }
template <typename... A> inline DBoptlist* DBMakeOptlist(A...) { return nullptr; }
template <typename... A> inline int DBClose(A...) { return -1; }
template <typename... A> inline int DBFreeOptlist(A...) { return -1; }
template <typename... A> inline int DBAddOption(A...) { return -1; }
template <typename... A> inline int DBMkDir(A...) { return -1; }
template <typename... A> inline int DBSetDir(A...) { return -1; }
template <typename... A> inline int DBSetCompression(A...) { return -1; }
template <typename... A> inline int DBWrite(A...) { return -1; }
template <typename... A> inline int DBPutQuadmesh(A...) { return -1; }
template <typename... A> inline int DBPutQuadvar(A...) { return -1; }
template <typename... A> inline int DBPutQuadvar1(A...) { return -1; }
template <typename... A> inline int DBPutMultimesh(A...) { return -1; }
template <typename... A> inline int DBPutMultivar(A...) { return -1; }

#endif
