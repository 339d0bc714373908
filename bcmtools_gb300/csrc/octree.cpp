// octree.cpp -- host-side octree of blocks: root grid, dividers, 2:1 face
// balancing, leaf orderings and per-leaf neighbour tables.
//
// Replaces the reference's Utils octree (BCMOctree.cpp, RootGrid.h, Node.h,
// Pedigree.h, SimpleDivider.h, SphereDivider.h, CylinderDivider.h, Partition.h
// for one rank).
// Semantics kept alike, because the neighbour tables and block ids must match
// the reference's for the same leaves:
//   * Z order and the reference's Hilbert order (BCMOctree.cpp:248-262);
//   * pedigree packing x:16 y:16 z:16 root:12 level:4 (Pedigree.h:52-60);
//   * child index x + 2y + 4z (Pedigree.h:96-107);
//   * neighbour search at the same level with root wrap-around, stopping at
//     the first leaf (BCMOctree.cpp:277-364);
//   * level differences -1/0/+1 and subface numbering, incl. the (z,x)
//     in-plane order of Y faces (NeighborInfo.h:176-211, BCMOctree.cpp:423-478);
//     levels two or more coarser are not neighbours (the reference skips them).
// The subface tables are derived here from the face geometry rather than
// tabulated.  Unlike the reference, building can balance the tree 2:1 across
// faces, and a violation is reported as an error instead of exit().
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bcmg.h"

namespace {

struct Node {
  uint64_t ped;
  int child0;  // index of first child (children contiguous), -1 for a leaf
  bool active;
};

inline uint64_t ped_make(unsigned level, unsigned x, unsigned y, unsigned z, unsigned root) {
  return ((uint64_t)x << 48) | ((uint64_t)y << 32) | ((uint64_t)z << 16) |
         ((uint64_t)root << 4) | (uint64_t)level;
}
inline unsigned ped_level(uint64_t p) { return p & 0xf; }
inline unsigned ped_x(uint64_t p) { return (p >> 48) & 0xffff; }
inline unsigned ped_y(uint64_t p) { return (p >> 32) & 0xffff; }
inline unsigned ped_z(uint64_t p) { return (p >> 16) & 0xffff; }
inline unsigned ped_root(uint64_t p) { return (p >> 4) & 0xfff; }
inline unsigned ped_child_at(uint64_t p, unsigned level) {
  unsigned sh = ped_level(p) - level;
  return ((ped_x(p) >> sh) & 1) | (((ped_y(p) >> sh) & 1) << 1) | (((ped_z(p) >> sh) & 1) << 2);
}

// In-plane axes of a face, in subface order: (origin0 axis, origin1 axis).
// X faces: (y, z); Y faces: (z, x); Z faces: (x, y)  (Scalar3DUpdater.h:527-584).
inline void face_plane_axes(int face, int* a0, int* a1) {
  int ax = face / 2;
  if (ax == 0) { *a0 = 1; *a1 = 2; }
  else if (ax == 1) { *a0 = 2; *a1 = 0; }
  else { *a0 = 0; *a1 = 1; }
}
// Subface of child `cid` as seen across `face` (NeighborInfo::childIdToSubface).
inline int child_to_subface(int face, int cid) {
  int a0, a1;
  face_plane_axes(face, &a0, &a1);
  return ((cid >> a0) & 1) | (((cid >> a1) & 1) << 1);
}
// Child of the neighbour touching `face` at `subface` (getNeighborChildId):
// the neighbour lies on the minus side for *_M faces, so its children with
// normal bit 1 touch us.
inline int neighbor_child(int face, int subface) {
  int ax = face / 2, a0, a1;
  face_plane_axes(face, &a0, &a1);
  int nb = (face % 2 == 0) ? 1 : 0;
  return (nb << ax) | ((subface & 1) << a0) | (((subface >> 1) & 1) << a1);
}

}  // namespace

struct bcmg_octree_s {
  bcmg_rootgrid rg;
  std::vector<Node> nodes;  // roots first (index = root id)
  std::vector<int> leaves;  // active leaves in block-id order
  std::vector<int> block_of;  // node -> block id (-1 if not an active leaf)
  std::string err;

  int nroot() const { return rg.nx * rg.ny * rg.nz; }
  int rx(int r) const { return r % rg.nx; }
  int ry(int r) const { return (r / rg.nx) % rg.ny; }
  int rz(int r) const { return (r / rg.nx) / rg.ny; }

  void split(int n) {
    uint64_t p = nodes[n].ped;
    int c0 = (int)nodes.size();
    nodes[n].child0 = c0;
    bool act = nodes[n].active;
    unsigned l = ped_level(p) + 1;
    for (int c = 0; c < 8; c++) {
      Node ch;
      ch.ped = ped_make(l, ped_x(p) * 2 + (c & 1), ped_y(p) * 2 + ((c >> 1) & 1),
                        ped_z(p) * 2 + ((c >> 2) & 1), ped_root(p));
      ch.child0 = -1;
      ch.active = act;
      nodes.push_back(ch);
    }
  }

  // Root neighbour across a face (RootGrid::getNeighborRoot, RootGrid.h), -1 if none.
  int neighbor_root(int r, int face) const {
    int i[3] = {rx(r), ry(r), rz(r)};
    int n[3] = {rg.nx, rg.ny, rg.nz};
    int ax = face / 2;
    i[ax] += (face % 2 == 0) ? -1 : 1;
    if (i[ax] < 0 || i[ax] >= n[ax]) {
      if (!((rg.periodic_mask >> ax) & 1)) return -1;
      i[ax] = (i[ax] + n[ax]) % n[ax];
    }
    return i[0] + rg.nx * (i[1] + rg.ny * i[2]);
  }

  bool on_outer(uint64_t p, int face) const {
    int ax = face / 2;
    unsigned c = ax == 0 ? ped_x(p) : ax == 1 ? ped_y(p) : ped_z(p);
    int r = ped_root(p);
    int ri = ax == 0 ? rx(r) : ax == 1 ? ry(r) : rz(r);
    int rn = ax == 0 ? rg.nx : ax == 1 ? rg.ny : rg.nz;
    unsigned mx = (1u << ped_level(p)) - 1;
    if (face % 2 == 0) return c == 0 && ri == 0;
    return c == mx && ri == rn - 1;
  }

  // Deepest node (up to the node's own level) at the same-level position
  // across `face`; -1 across a non-periodic outer boundary
  // (BCMOctree::findNeighborNode, BCMOctree.cpp:277-364).
  int find_neighbor(int n, int face) const {
    uint64_t p = nodes[n].ped;
    unsigned l = ped_level(p);
    long c[3] = {ped_x(p), ped_y(p), ped_z(p)};
    long mx = (1L << l) - 1;
    int r = ped_root(p);
    int ax = face / 2;
    c[ax] += (face % 2 == 0) ? -1 : 1;
    if (c[ax] < 0 || c[ax] > mx) {
      r = neighbor_root(r, face);
      if (r < 0) return -1;
      c[ax] = (c[ax] < 0) ? mx : 0;
    }
    uint64_t q = ped_make(l, (unsigned)c[0], (unsigned)c[1], (unsigned)c[2], r);
    int cur = r;
    for (unsigned lv = 1; lv <= l; lv++) {
      if (nodes[cur].child0 < 0) break;
      cur = nodes[cur].child0 + (int)ped_child_at(q, lv);
    }
    return cur;
  }

  // Box of a node in physical coordinates.
  void box(uint64_t p, double lo[3], double hi[3]) const {
    int r = ped_root(p);
    double d = rg.root_length / (double)(1u << ped_level(p));
    double ri[3] = {(double)rx(r), (double)ry(r), (double)rz(r)};
    unsigned c[3] = {ped_x(p), ped_y(p), ped_z(p)};
    for (int a = 0; a < 3; a++) {
      lo[a] = rg.origin[a] + ri[a] * rg.root_length + c[a] * d;
      hi[a] = lo[a] + d;
    }
  }

  enum { BRANCH, LEAF_ACTIVE, LEAF_INACTIVE };

  int divide(const bcmg_divider& dv, uint64_t p) const {
    int level = (int)ped_level(p);
    switch (dv.kind) {
      case BCMG_DIV_FLAT:  // FlatDivider (SimpleDivider.h:30-64)
        return level >= dv.max_level ? LEAF_ACTIVE : BRANCH;
      case BCMG_DIV_SIMPLE: {  // SimpleDivider (SimpleDivider.h:67-150)
        if (level < dv.min_level) return BRANCH;
        if (level >= dv.max_level) return LEAF_ACTIVE;
        int mask = dv.direction_mask ? dv.direction_mask : 63;
        for (int f = 0; f < 6; f++)
          if (((mask >> f) & 1) && on_outer_root_side(p, f)) return BRANCH;
        return LEAF_ACTIVE;
      }
      case BCMG_DIV_SPHERE_SURFACE: {
        if (level < dv.min_level) return BRANCH;
        if (level >= dv.max_level) return LEAF_ACTIVE;
        double lo[3], hi[3], dmin = 0, dmax = 0;
        box(p, lo, hi);
        for (int a = 0; a < 3; a++) {
          double c = dv.center[a];
          double e = c < lo[a] ? lo[a] - c : (c > hi[a] ? c - hi[a] : 0.0);
          double f = std::max(std::fabs(c - lo[a]), std::fabs(c - hi[a]));
          dmin += e * e;
          dmax += f * f;
        }
        double r2 = dv.radius * dv.radius;
        return (dmin <= r2 && r2 <= dmax) ? BRANCH : LEAF_ACTIVE;
      }
      case BCMG_DIV_SPHERE:  // SphereDivider (SphereDivider.h:28-150), REAL_TYPE float
        return sphere_divide(dv, p, false);
      case BCMG_DIV_CYLINDER:  // CylinderDivider (CylinderDivider.h:28-153)
        return sphere_divide(dv, p, true);
      case BCMG_DIV_BALLS: {
        if (level < dv.min_level) return BRANCH;
        if (level >= dv.max_level) return LEAF_ACTIVE;
        double lo[3], hi[3];
        box(p, lo, hi);
        double r2 = dv.radius * dv.radius;
        for (int q = 0; q < dv.npoints; q++) {
          double dmin = 0;
          for (int a = 0; a < 3; a++) {
            double c = dv.points[3 * q + a];
            double e = c < lo[a] ? lo[a] - c : (c > hi[a] ? c - hi[a] : 0.0);
            dmin += e * e;
          }
          if (dmin <= r2) return BRANCH;
        }
        return LEAF_ACTIVE;
      }
    }
    return LEAF_ACTIVE;
  }

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
  int sphere_divide(const bcmg_divider& dv, uint64_t p, bool cylinder) const {
    const int dims = cylinder ? 2 : 3;
    const int level = (int)ped_level(p);
    if (level < dv.min_level) return BRANCH;
    const int r = ped_root(p);
    const int ri[3] = {rx(r), ry(r), rz(r)};
    const int pc[3] = {(int)ped_x(p), (int)ped_y(p), (int)ped_z(p)};
    const int max0 = (1 << level) - 1;
    const float d = (float)(1.0 / (max0 + 1));
    float lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
      lo[a] = (float)ri[a] + (float)pc[a] * d;
      hi[a] = (float)ri[a] + (float)(pc[a] + 1) * d;
    }
    if (level < dv.max_level) {
      const int n = 1 << (dv.max_level - level - 1);
      const float dd = d * (float)(n - 1) / (float)n;
      for (int a = 0; a < 3; a++) {
        if (!on_outer(p, 2 * a)) lo[a] -= dd;
        if (!on_outer(p, 2 * a + 1)) hi[a] += dd;
      }
    }
    const float len = 1.0f, org = 0.0f;  // MultiRootDivider(Vec3r(0,0,0), 1.0, rootGrid)
    const float margin = (float)dv.margin_ratio / (float)(1 << dv.max_level);
    float o[3], rr = (float)dv.radius;
    for (int a = 0; a < 3; a++) {
      lo[a] = org + lo[a] * len;
      hi[a] = org + hi[a] * len;
      lo[a] = lo[a] - margin;  // extra margin (SphereDivider.h:88-89)
      hi[a] = hi[a] + margin;
      o[a] = (float)dv.center[a];
    }
    const float r2 = rr * rr;
    // wholly inside: the farthest point is closer than r (checkInner)
    bool inner = true;
    float far2 = 0.0f;
    for (int a = 0; a < dims && inner; a++) {
      const float e = std::max(std::fabs(lo[a] - o[a]), std::fabs(hi[a] - o[a]));
      far2 += e * e;
      if (far2 >= r2) inner = false;
    }
    if (inner) return cylinder ? LEAF_ACTIVE : LEAF_INACTIVE;
    // wholly outside: the nearest point is at r or beyond (checkOuter)
    float near2 = 0.0f;
    for (int a = 0; a < dims; a++) {
      float e = 0.0f;
      if (o[a] < lo[a]) e = lo[a] - o[a];
      else if (o[a] > hi[a]) e = o[a] - hi[a];
      near2 += e * e;
      if (near2 >= r2) return cylinder ? LEAF_INACTIVE : LEAF_ACTIVE;
    }
    return level == dv.max_level ? LEAF_ACTIVE : BRANCH;
  }

  // SimpleDivider's test: node touches the outer face of the root grid.
  bool on_outer_root_side(uint64_t p, int face) const { return on_outer(p, face); }

  void build_by_divider(const bcmg_divider& dv) {
    std::vector<int> stack;
    for (int r = nroot() - 1; r >= 0; r--) stack.push_back(r);
    while (!stack.empty()) {
      int n = stack.back();
      stack.pop_back();
      int t = divide(dv, nodes[n].ped);
      if (t == LEAF_ACTIVE) continue;
      if (t == LEAF_INACTIVE) { nodes[n].active = false; continue; }
      if ((int)ped_level(nodes[n].ped) >= 15) continue;
      split(n);
      int c0 = nodes[n].child0;
      for (int c = 7; c >= 0; c--) stack.push_back(c0 + c);
    }
  }

  // 2:1 face balance: refine any leaf two or more levels coarser than a
  // face neighbour, until none remains.
  void balance() {
    for (;;) {
      std::vector<int> mark;
      std::vector<char> marked(nodes.size(), 0);
      for (int n = 0; n < (int)nodes.size(); n++) {
        if (nodes[n].child0 >= 0) continue;
        unsigned l = ped_level(nodes[n].ped);
        if (l < 2) continue;
        for (int f = 0; f < 6; f++) {
          int m = find_neighbor(n, f);
          if (m < 0) continue;
          if (nodes[m].child0 < 0 && ped_level(nodes[m].ped) + 1 < l && !marked[m]) {
            marked[m] = 1;
            mark.push_back(m);
          }
        }
      }
      if (mark.empty()) break;
      for (int m : mark) split(m);
    }
  }

  void collect_z(int n) {
    if (nodes[n].child0 < 0) {
      if (nodes[n].active) leaves.push_back(n);
      return;
    }
    for (int c = 0; c < 8; c++) collect_z(nodes[n].child0 + c);
  }

  // Hilbert order of the reference (BCMOctree.cpp:248-262 with its
  // orientation tables): a self-similar curve.  A frame maps the base visit
  // order of the eight children -- the Gray code 0,1,3,2,6,7,5,4 of the child
  // index x + 2y + 4z -- onto child indices by an axis permutation and a
  // reflection; the k-th visited child's frame is its parent's frame after
  // kHilbertStep[k].  The eight steps were fitted to the reference's leaf
  // orders (its sor2 example mesh and a two-root sphere mesh) and reproduce
  // them exactly.
  struct Frame {
    uint8_t to[3];  // input axis a goes to axis to[a]
    uint8_t flip;   // then these axes are reflected
  };
  static unsigned frame_apply(const Frame& f, unsigned v) {
    unsigned o = 0;
    for (int a = 0; a < 3; a++)
      if ((v >> a) & 1) o |= 1u << f.to[a];
    return o ^ f.flip;
  }
  // outer after inner
  static Frame frame_compose(const Frame& outer, const Frame& inner) {
    Frame r;
    for (int a = 0; a < 3; a++) r.to[a] = outer.to[inner.to[a]];
    r.flip = (uint8_t)frame_apply(outer, inner.flip) ^ (uint8_t)frame_apply(outer, 0) ^
             outer.flip;
    return r;
  }
  void collect_hilbert(int n, const Frame& f) {
    static const unsigned kGray[8] = {0, 1, 3, 2, 6, 7, 5, 4};
    static const Frame kHilbertStep[8] = {
        {{2, 1, 0}, 0}, {{0, 2, 1}, 0}, {{0, 1, 2}, 0}, {{2, 0, 1}, 5},
        {{2, 0, 1}, 3}, {{0, 1, 2}, 0}, {{0, 2, 1}, 6}, {{2, 1, 0}, 5}};
    if (nodes[n].child0 < 0) {
      if (nodes[n].active) leaves.push_back(n);
      return;
    }
    for (int k = 0; k < 8; k++)
      collect_hilbert(nodes[n].child0 + (int)frame_apply(f, kGray[k]),
                      frame_compose(f, kHilbertStep[k]));
  }

  void order(int ordering, uint64_t seed) {
    leaves.clear();
    if (ordering == BCMG_ORDER_HILBERT) {
      const Frame identity = {{0, 1, 2}, 0};
      for (int r = 0; r < nroot(); r++) collect_hilbert(r, identity);
    } else {
      for (int r = 0; r < nroot(); r++) collect_z(r);
    }
    if (ordering == BCMG_ORDER_RANDOM) {
      uint64_t s = seed;
      for (size_t i = leaves.size(); i > 1; i--) {
        s += 0x9E3779B97F4A7C15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        std::swap(leaves[i - 1], leaves[z % i]);
      }
    }
    block_of.assign(nodes.size(), -1);
    for (size_t i = 0; i < leaves.size(); i++) block_of[leaves[i]] = (int)i;
  }
};

static bool valid_rg(const bcmg_rootgrid* rg) {
  return rg && rg->nx > 0 && rg->ny > 0 && rg->nz > 0 &&
         (long)rg->nx * rg->ny * rg->nz <= 0xfff + 1 && rg->root_length > 0;
}

extern "C" {

BCMG_API int bcmg_octree_build(bcmg_octree* out, const bcmg_rootgrid* rg,
                               const bcmg_divider* div, int ordering, uint64_t seed) {
  if (!out || !valid_rg(rg) || !div) return BCMG_USAGE;
  if (div->max_level < 0 || div->max_level > 15 || div->min_level < 0 ||
      div->min_level > div->max_level)
    return BCMG_USAGE;
  if (div->kind == BCMG_DIV_BALLS && div->npoints > 0 && !div->points) return BCMG_USAGE;
  if (ordering < 0 || ordering > BCMG_ORDER_RANDOM) return BCMG_USAGE;
  bcmg_octree t = new (std::nothrow) bcmg_octree_s;
  if (!t) return BCMG_MEMORY;
  t->rg = *rg;
  for (int r = 0; r < t->nroot(); r++) t->nodes.push_back(Node{ped_make(0, 0, 0, 0, r), -1, true});
  t->build_by_divider(*div);
  if (div->balance) t->balance();
  t->order(ordering, seed);
  *out = t;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_octree_from_pedigrees(bcmg_octree* out, const bcmg_rootgrid* rg,
                                        const uint64_t* peds, int n) {
  if (!out || !valid_rg(rg) || (n > 0 && !peds) || n < 0) return BCMG_USAGE;
  bcmg_octree t = new (std::nothrow) bcmg_octree_s;
  if (!t) return BCMG_MEMORY;
  t->rg = *rg;
  for (int r = 0; r < t->nroot(); r++) t->nodes.push_back(Node{ped_make(0, 0, 0, 0, r), -1, true});
  // Building from a pedigree list (BCMOctree.cpp:66-96): siblings created on
  // the way down start inactive; listed leaves become active, in list order.
  std::vector<int> order;
  for (int i = 0; i < n; i++) {
    uint64_t p = peds[i];
    unsigned root = ped_root(p), l = ped_level(p);
    if ((int)root >= t->nroot() || l > 15) { delete t; return BCMG_USAGE; }
    int cur = (int)root;
    for (unsigned lv = 1; lv <= l; lv++) {
      if (t->nodes[cur].child0 < 0) {
        t->split(cur);
        for (int c = 0; c < 8; c++) t->nodes[t->nodes[cur].child0 + c].active = false;
      }
      cur = t->nodes[cur].child0 + (int)ped_child_at(p, lv);
    }
    if (t->nodes[cur].child0 >= 0) { delete t; return BCMG_USAGE; }
    t->nodes[cur].active = true;
    order.push_back(cur);
  }
  t->leaves = order;
  t->block_of.assign(t->nodes.size(), -1);
  for (size_t i = 0; i < order.size(); i++) {
    if (t->block_of[order[i]] >= 0) { delete t; return BCMG_USAGE; }  // duplicate
    t->block_of[order[i]] = (int)i;
  }
  *out = t;
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_octree_num_leaves(bcmg_octree t, int* n) {
  if (!t || !n) return BCMG_USAGE;
  *n = (int)t->leaves.size();
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_octree_leaves(bcmg_octree t, uint64_t* ped, int* level, double* origin,
                                double* block_size) {
  if (!t) return BCMG_USAGE;
  for (size_t i = 0; i < t->leaves.size(); i++) {
    uint64_t p = t->nodes[t->leaves[i]].ped;
    if (ped) ped[i] = p;
    if (level) level[i] = (int)ped_level(p);
    double lo[3], hi[3];
    t->box(p, lo, hi);
    if (origin) for (int a = 0; a < 3; a++) origin[3 * i + a] = lo[a];
    if (block_size) block_size[i] = t->rg.root_length / (double)(1u << ped_level(p));
  }
  return BCMG_SUCCESS;
}

BCMG_API int bcmg_octree_neighbors(bcmg_octree t, int* ld, int* id, int* sf, int* outer) {
  if (!t || !ld || !id || !sf) return BCMG_USAGE;
  int nb = (int)t->leaves.size();
  for (int b = 0; b < nb; b++) {
    int n = t->leaves[b];
    uint64_t p = t->nodes[n].ped;
    int l = (int)ped_level(p);
    for (int f = 0; f < 6; f++) {
      int k = b * 6 + f;
      ld[k] = 0;
      sf[k] = 0;
      for (int s = 0; s < 4; s++) id[k * 4 + s] = -1;
      if (outer) outer[k] = t->on_outer(p, f) ? 1 : 0;
      int m = t->find_neighbor(n, f);
      if (m < 0) continue;
      int diff = (int)ped_level(t->nodes[m].ped) - l;
      if (diff == -1) {
        if (!t->nodes[m].active) continue;
        ld[k] = -1;
        id[k * 4] = t->block_of[m];
        sf[k] = child_to_subface(f, (int)ped_child_at(p, (unsigned)l));
      } else if (diff == 0) {
        if (t->nodes[m].child0 < 0) {
          if (!t->nodes[m].active) continue;
          id[k * 4] = t->block_of[m];
        } else {
          ld[k] = 1;
          for (int s = 0; s < 4; s++) {
            int ch = t->nodes[m].child0 + neighbor_child(f, s);
            if (t->nodes[ch].child0 >= 0) return BCMG_FAILURE;  // 2:1 broken
            if (!t->nodes[ch].active) continue;
            id[k * 4 + s] = t->block_of[ch];
          }
        }
      }
    }
  }
  return BCMG_SUCCESS;
}

BCMG_API void bcmg_octree_destroy(bcmg_octree t) { delete t; }

}  // extern "C"
