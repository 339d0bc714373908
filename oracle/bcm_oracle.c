/*
 * bcm_oracle.c -- CPU restatement of the BCMTools ghost-update and stencil
 * path.  TEST INFRASTRUCTURE ONLY (see bcm_oracle.h); never part of the
 * product.  Compiled twice over bcm_oracle_impl.inc: once with T = float (the
 * reference built with real_type=float) and once with T = double.
 */
#include "bcm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int bcmo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads of the following parallel loops; 1 makes every sum over blocks
 * run in block order (what a single-threaded reference run does). */
void bcmo_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

/* ---- face list (BlockManager::setFaceLists, BlockManager.cpp:471-510) ---- */
typedef struct { int id, face, subface; } face_id;

static int face_axis(int face) { return face / 2; }

/* Builds the local face list: level difference 0/-1 -> one entry per face,
 * +1 -> one entry per existing subface.  Returns the entry count; *out is
 * malloc'ed.  A face is local when its neighbour exists (single rank). */
static int build_face_list(const bcmo_mesh* m, int axis_mask, int ld_mask, face_id** out) {
  int cap = m->nb * 24 + 1, n = 0;
  face_id* fl = (face_id*)malloc(sizeof(face_id) * cap);
  for (int b = 0; b < m->nb; b++) {
    for (int f = 0; f < 6; f++) {
      int ld = m->nbr_ld[b * 6 + f];
      if (!((axis_mask >> face_axis(f)) & 1)) continue;
      if (!((ld_mask >> (ld + 1)) & 1)) continue;
      if (ld == 0 || ld == -1) {
        if (m->nbr_id[(b * 6 + f) * 4 + 0] >= 0) {
          fl[n].id = b; fl[n].face = f; fl[n].subface = 0; n++;
        }
      } else if (ld == 1) {
        for (int s = 0; s < 4; s++) {
          if (m->nbr_id[(b * 6 + f) * 4 + s] >= 0) {
            fl[n].id = b; fl[n].face = f; fl[n].subface = s; n++;
          }
        }
      }
    }
  }
  *out = fl;
  return n;
}

/* VCUpdater::subfaceOrigin0/1 (VCUpdater.h:252-273). */
static int sf_origin0(int sf) { return sf & 1; }
static int sf_origin1(int sf) { return (sf >> 1) & 1; }

/* C2F parameters (Scalar3DUpdater.h:242-266): I = min(max(i/2-1+i%2,0),n-2),
 * r = -0.25 + 0.5 i - I.  All values are multiples of 1/4, so the result is
 * exact in float and in double. */
static void lin_interp(int i, int n, int* I, double* r) {
  int v = i / 2 - 1 + i % 2;
  if (v < 0) v = 0;
  if (v > n - 2) v = n - 2;
  *I = v;
  *r = -0.25 + 0.5 * i - (double)v;
}

#define T float
#define SFX f32
#define RPROD(r, c) ((double)((float)(r) * (c)))
#include "bcm_oracle_impl.inc"
#undef T
#undef SFX
#undef RPROD

#define T double
#define SFX f64
#define RPROD(r, c) ((r) * (c))
#include "bcm_oracle_impl.inc"
#undef T
#undef SFX
#undef RPROD
