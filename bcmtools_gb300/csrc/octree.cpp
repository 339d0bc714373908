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
#include "octree_div.h"

using namespace bcmg_oct;

namespace {

struct Node {
  uint64_t ped;
  int child0;  // index of first child (children contiguous), -1 for a leaf
  bool active;
};

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

  int neighbor_root(int r, int face) const { return bcmg_oct::neighbor_root(rg, r, face); }
  bool on_outer(uint64_t p, int face) const { return bcmg_oct::on_outer(rg, p, face); }

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

  void box(uint64_t p, double lo[3], double hi[3]) const { bcmg_oct::box(rg, p, lo, hi); }

  void build_by_divider(const bcmg_divider& dv) {
    std::vector<int> stack;
    for (int r = nroot() - 1; r >= 0; r--) stack.push_back(r);
    while (!stack.empty()) {
      int n = stack.back();
      stack.pop_back();
      int t = bcmg_oct::divide(rg, dv, nodes[n].ped);
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
