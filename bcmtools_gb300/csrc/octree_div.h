// octree_div.h -- pedigree packing, root-grid geometry and the dividers as
// functions of one node, shared by the host octree builder (octree.cpp) and
// the device mesh set-up (mesh_dev.cu), so that both decide every node alike.
//
// Reference: Pedigree.h:52-60 (packing x:16 y:16 z:16 root:12 level:4),
// Pedigree.h:96-107 (child index x + 2y + 4z), RootGrid.h (root neighbours,
// outer faces), SimpleDivider.h, SphereDivider.h, CylinderDivider.h,
// MultiRootDivider.h:56-100 (search region).
//
// Arithmetic goes through the f_* / d_* helpers: round-to-nearest operations
// without multiply-add contraction on the device, and plain operators on the
// host, whose translation unit is compiled with -ffp-contract=off.
#pragma once
#include <cstdint>

#include "bcmg.h"

#ifdef __CUDACC__
#define BCMG_HD __host__ __device__ __forceinline__
#else
#define BCMG_HD inline
#endif

namespace bcmg_oct {

BCMG_HD uint64_t ped_make(unsigned level, unsigned x, unsigned y, unsigned z, unsigned root) {
  return ((uint64_t)x << 48) | ((uint64_t)y << 32) | ((uint64_t)z << 16) |
         ((uint64_t)root << 4) | (uint64_t)level;
}
BCMG_HD unsigned ped_level(uint64_t p) { return (unsigned)(p & 0xf); }
BCMG_HD unsigned ped_x(uint64_t p) { return (unsigned)((p >> 48) & 0xffff); }
BCMG_HD unsigned ped_y(uint64_t p) { return (unsigned)((p >> 32) & 0xffff); }
BCMG_HD unsigned ped_z(uint64_t p) { return (unsigned)((p >> 16) & 0xffff); }
BCMG_HD unsigned ped_root(uint64_t p) { return (unsigned)((p >> 4) & 0xfff); }
// Child index of p's ancestor at `level` within its parent (x + 2y + 4z).
BCMG_HD unsigned ped_child_at(uint64_t p, unsigned level) {
  const unsigned sh = ped_level(p) - level;
  return ((ped_x(p) >> sh) & 1) | (((ped_y(p) >> sh) & 1) << 1) | (((ped_z(p) >> sh) & 1) << 2);
}

BCMG_HD int rg_nroot(const bcmg_rootgrid& rg) { return rg.nx * rg.ny * rg.nz; }
BCMG_HD int rg_x(const bcmg_rootgrid& rg, int r) { return r % rg.nx; }
BCMG_HD int rg_y(const bcmg_rootgrid& rg, int r) { return (r / rg.nx) % rg.ny; }
BCMG_HD int rg_z(const bcmg_rootgrid& rg, int r) { return (r / rg.nx) / rg.ny; }

// Root neighbour across a face (RootGrid::getNeighborRoot), -1 if none.
BCMG_HD int neighbor_root(const bcmg_rootgrid& rg, int r, int face) {
  int i[3] = {rg_x(rg, r), rg_y(rg, r), rg_z(rg, r)};
  const int n[3] = {rg.nx, rg.ny, rg.nz};
  const int ax = face / 2;
  i[ax] += (face % 2 == 0) ? -1 : 1;
  if (i[ax] < 0 || i[ax] >= n[ax]) {
    if (!((rg.periodic_mask >> ax) & 1)) return -1;
    i[ax] = (i[ax] + n[ax]) % n[ax];
  }
  return i[0] + rg.nx * (i[1] + rg.ny * i[2]);
}

// Node on the outer face `face` of the root grid (checkOnOuterBoundary).
BCMG_HD bool on_outer(const bcmg_rootgrid& rg, uint64_t p, int face) {
  const int ax = face / 2;
  const unsigned c = ax == 0 ? ped_x(p) : ax == 1 ? ped_y(p) : ped_z(p);
  const int r = (int)ped_root(p);
  const int ri = ax == 0 ? rg_x(rg, r) : ax == 1 ? rg_y(rg, r) : rg_z(rg, r);
  const int rn = ax == 0 ? rg.nx : ax == 1 ? rg.ny : rg.nz;
  const unsigned mx = (1u << ped_level(p)) - 1;
  if (face % 2 == 0) return c == 0 && ri == 0;
  return c == mx && ri == rn - 1;
}

#ifdef __CUDA_ARCH__
BCMG_HD float f_add(float a, float b) { return __fadd_rn(a, b); }
BCMG_HD float f_sub(float a, float b) { return __fsub_rn(a, b); }
BCMG_HD float f_mul(float a, float b) { return __fmul_rn(a, b); }
BCMG_HD double d_add(double a, double b) { return __dadd_rn(a, b); }
BCMG_HD double d_sub(double a, double b) { return __dsub_rn(a, b); }
BCMG_HD double d_mul(double a, double b) { return __dmul_rn(a, b); }
#else
BCMG_HD float f_add(float a, float b) { return a + b; }
BCMG_HD float f_sub(float a, float b) { return a - b; }
BCMG_HD float f_mul(float a, float b) { return a * b; }
BCMG_HD double d_add(double a, double b) { return a + b; }
BCMG_HD double d_sub(double a, double b) { return a - b; }
BCMG_HD double d_mul(double a, double b) { return a * b; }
#endif
BCMG_HD float f_abs(float a) { return a < 0.0f ? -a : a; }
BCMG_HD double d_abs(double a) { return a < 0.0 ? -a : a; }
BCMG_HD float f_max(float a, float b) { return a < b ? b : a; }
BCMG_HD double d_max(double a, double b) { return a < b ? b : a; }

// Box of a node in physical coordinates.
BCMG_HD void box(const bcmg_rootgrid& rg, uint64_t p, double lo[3], double hi[3]) {
  const int r = (int)ped_root(p);
  const double d = rg.root_length / (double)(1u << ped_level(p));
  const double ri[3] = {(double)rg_x(rg, r), (double)rg_y(rg, r), (double)rg_z(rg, r)};
  const unsigned c[3] = {ped_x(p), ped_y(p), ped_z(p)};
  for (int a = 0; a < 3; a++) {
    lo[a] = d_add(d_add(rg.origin[a], d_mul(ri[a], rg.root_length)), d_mul((double)c[a], d));
    hi[a] = d_add(lo[a], d);
  }
}

enum { BRANCH = 0, LEAF_ACTIVE = 1, LEAF_INACTIVE = 2 };

// SphereDivider: blocks wholly inside the sphere become inactive leaves,
// blocks wholly outside stay leaves, the rest divide down to max_level.
// CylinderDivider (`cylinder`): the same tests on x and y only, around the
// axis through (center[0], center[1]) along z, with the roles swapped --
// blocks wholly inside stay leaves, blocks wholly outside become inactive.
// The search box is MultiRootDivider::defineSearchRegion
// (MultiRootDivider.h:56-100): the block widened on every side that is not
// the root grid's outer side by d(n-1)/n, n = 2^(max_level - level - 1)
// (the reference's ripple margin), then scaled by the root length and moved
// to the origin.  The reference's SphereDivider and CylinderDivider build
// that MultiRootDivider with origin (0,0,0) and root length 1
// (SphereDivider.h:72, CylinderDivider.h:69) whatever the mesh's root grid
// is, so their boxes -- and the center and radius they are tested against --
// are in root-index units (unit root blocks, root 0 at the origin), and so
// are they here.  Arithmetic in float, the reference's default REAL_TYPE,
// in its operation order, so that boxes that touch the sphere decide alike.
BCMG_HD int sphere_divide(const bcmg_rootgrid& rg, const bcmg_divider& dv, uint64_t p,
                          bool cylinder) {
  const int dims = cylinder ? 2 : 3;
  const int level = (int)ped_level(p);
  if (level < dv.min_level) return BRANCH;
  const int r = (int)ped_root(p);
  const int ri[3] = {rg_x(rg, r), rg_y(rg, r), rg_z(rg, r)};
  const int pc[3] = {(int)ped_x(p), (int)ped_y(p), (int)ped_z(p)};
  const int max0 = (1 << level) - 1;
  const float d = (float)(1.0 / (max0 + 1));
  float lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = f_add((float)ri[a], f_mul((float)pc[a], d));
    hi[a] = f_add((float)ri[a], f_mul((float)(pc[a] + 1), d));
  }
  if (level < dv.max_level) {
    const int n = 1 << (dv.max_level - level - 1);
    const float dd = f_mul(d, (float)(n - 1)) / (float)n;
    for (int a = 0; a < 3; a++) {
      if (!on_outer(rg, p, 2 * a)) lo[a] = f_sub(lo[a], dd);
      if (!on_outer(rg, p, 2 * a + 1)) hi[a] = f_add(hi[a], dd);
    }
  }
  const float len = 1.0f, org = 0.0f;  // MultiRootDivider(Vec3r(0,0,0), 1.0, rootGrid)
  const float margin = (float)dv.margin_ratio / (float)(1 << dv.max_level);
  float o[3];
  const float rr = (float)dv.radius;
  for (int a = 0; a < 3; a++) {
    lo[a] = f_add(org, f_mul(lo[a], len));
    hi[a] = f_add(org, f_mul(hi[a], len));
    lo[a] = f_sub(lo[a], margin);  // extra margin (SphereDivider.h:88-89)
    hi[a] = f_add(hi[a], margin);
    o[a] = (float)dv.center[a];
  }
  const float r2 = f_mul(rr, rr);
  // wholly inside: the farthest point is closer than r (checkInner)
  bool inner = true;
  float far2 = 0.0f;
  for (int a = 0; a < dims && inner; a++) {
    const float e = f_max(f_abs(f_sub(lo[a], o[a])), f_abs(f_sub(hi[a], o[a])));
    far2 = f_add(far2, f_mul(e, e));
    if (far2 >= r2) inner = false;
  }
  if (inner) return cylinder ? LEAF_ACTIVE : LEAF_INACTIVE;
  // wholly outside: the nearest point is at r or beyond (checkOuter)
  float near2 = 0.0f;
  for (int a = 0; a < dims; a++) {
    float e = 0.0f;
    if (o[a] < lo[a]) e = f_sub(lo[a], o[a]);
    else if (o[a] > hi[a]) e = f_sub(o[a], hi[a]);
    near2 = f_add(near2, f_mul(e, e));
    if (near2 >= r2) return cylinder ? LEAF_INACTIVE : LEAF_ACTIVE;
  }
  return level == dv.max_level ? LEAF_ACTIVE : BRANCH;
}

// The fate of node p under divider dv (Divider::operator(), the reference's
// dividers one by one).
BCMG_HD int divide(const bcmg_rootgrid& rg, const bcmg_divider& dv, uint64_t p) {
  const int level = (int)ped_level(p);
  switch (dv.kind) {
    case BCMG_DIV_FLAT:  // FlatDivider (SimpleDivider.h:30-64)
      return level >= dv.max_level ? LEAF_ACTIVE : BRANCH;
    case BCMG_DIV_SIMPLE: {  // SimpleDivider (SimpleDivider.h:67-150)
      if (level < dv.min_level) return BRANCH;
      if (level >= dv.max_level) return LEAF_ACTIVE;
      const int mask = dv.direction_mask ? dv.direction_mask : 63;
      for (int f = 0; f < 6; f++)
        if (((mask >> f) & 1) && on_outer(rg, p, f)) return BRANCH;
      return LEAF_ACTIVE;
    }
    case BCMG_DIV_SPHERE_SURFACE: {
      if (level < dv.min_level) return BRANCH;
      if (level >= dv.max_level) return LEAF_ACTIVE;
      double lo[3], hi[3], dmin = 0, dmax = 0;
      box(rg, p, lo, hi);
      for (int a = 0; a < 3; a++) {
        const double c = dv.center[a];
        const double e = c < lo[a] ? d_sub(lo[a], c) : (c > hi[a] ? d_sub(c, hi[a]) : 0.0);
        const double f = d_max(d_abs(d_sub(c, lo[a])), d_abs(d_sub(c, hi[a])));
        dmin = d_add(dmin, d_mul(e, e));
        dmax = d_add(dmax, d_mul(f, f));
      }
      const double r2 = d_mul(dv.radius, dv.radius);
      return (dmin <= r2 && r2 <= dmax) ? BRANCH : LEAF_ACTIVE;
    }
    case BCMG_DIV_SPHERE:  // SphereDivider (SphereDivider.h:28-150), REAL_TYPE float
      return sphere_divide(rg, dv, p, false);
    case BCMG_DIV_CYLINDER:  // CylinderDivider (CylinderDivider.h:28-153)
      return sphere_divide(rg, dv, p, true);
    case BCMG_DIV_BALLS: {
      if (level < dv.min_level) return BRANCH;
      if (level >= dv.max_level) return LEAF_ACTIVE;
      double lo[3], hi[3];
      box(rg, p, lo, hi);
      const double r2 = d_mul(dv.radius, dv.radius);
      for (int q = 0; q < dv.npoints; q++) {
        double dmin = 0;
        for (int a = 0; a < 3; a++) {
          const double c = dv.points[3 * q + a];
          const double e = c < lo[a] ? d_sub(lo[a], c) : (c > hi[a] ? d_sub(c, hi[a]) : 0.0);
          dmin = d_add(dmin, d_mul(e, e));
        }
        if (dmin <= r2) return BRANCH;
      }
      return LEAF_ACTIVE;
    }
  }
  return LEAF_ACTIVE;
}

// In-plane axes of a face, in subface order: (origin0 axis, origin1 axis).
// X faces: (y, z); Y faces: (z, x); Z faces: (x, y)  (Scalar3DUpdater.h:527-584).
BCMG_HD void face_plane_axes(int face, int* a0, int* a1) {
  const int ax = face / 2;
  if (ax == 0) { *a0 = 1; *a1 = 2; }
  else if (ax == 1) { *a0 = 2; *a1 = 0; }
  else { *a0 = 0; *a1 = 1; }
}
// Subface of child `cid` as seen across `face` (NeighborInfo::childIdToSubface).
BCMG_HD int child_to_subface(int face, int cid) {
  int a0, a1;
  face_plane_axes(face, &a0, &a1);
  return ((cid >> a0) & 1) | (((cid >> a1) & 1) << 1);
}
// Child of the neighbour touching `face` at `subface` (getNeighborChildId):
// the neighbour lies on the minus side for *_M faces, so its children with
// normal bit 1 touch us.
BCMG_HD int neighbor_child(int face, int subface) {
  const int ax = face / 2;
  int a0, a1;
  face_plane_axes(face, &a0, &a1);
  const int nb = (face % 2 == 0) ? 1 : 0;
  return (nb << ax) | ((subface & 1) << a0) | (((subface >> 1) & 1) << a1);
}

}  // namespace bcmg_oct
