/*
 * pvoracle.c -- CPU restatement of OpenPV's delivery + LCA path (test infrastructure only).
 *
 * This file is the oracle the GPU path is checked against; nothing in the product
 * links it.  Integer geometry lives here; the numeric loops are written once in
 * pvoracle_real.inc and instantiated for float (reference order, bit-faithful) and
 * double (the FP64 oracle).  Build with -ffp-contract=off so that no multiply-add is
 * fused: the reference CPU build on x86-64 has no FMA contraction either.
 */
#include "pvoracle.h"

#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* utils/conversions.hpp index helpers: k = (y*nx + x)*nf + f */
static inline int kxPos(int k, int nx, int ny, int nf) { (void)ny; return (k / nf) % nx; }
static inline int kyPos(int k, int nx, int ny, int nf) { (void)ny; return k / (nx * nf); }
static inline int featureIndex(int k, int nx, int ny, int nf) { (void)nx; (void)ny; return k % nf; }
static inline int kIndex(int x, int y, int f, int nx, int ny, int nf) { (void)ny; return (y * nx + x) * nf + f; }
/* utils/conversions.hpp:402-407 */
static inline int kIndexExtended(int k, int nx, int ny, int nf, int lt, int rt, int dn, int up) {
   int kx = lt + kxPos(k, nx, ny, nf);
   int ky = up + kyPos(k, nx, ny, nf);
   int kf = featureIndex(k, nx, ny, nf);
   return kIndex(kx, ky, kf, nx + lt + rt, ny + dn + up, nf);
}

static inline int loc_nx_ext(const pvo_loc *l) { return l->nx + l->halo.lt + l->halo.rt; }
static inline int loc_ny_ext(const pvo_loc *l) { return l->ny + l->halo.dn + l->halo.up; }
static inline int loc_num_ext(const pvo_loc *l) { return loc_nx_ext(l) * loc_ny_ext(l) * l->nf; }
static inline int loc_num_res(const pvo_loc *l) { return l->nx * l->ny * l->nf; }

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* utils/requiredConvolveMargin.hpp */
int pvo_required_margin(int nPre, int nPost, int patchSize) {
   if (nPre == nPost) {
      if (patchSize % 2 != 1) return -1;
      return (patchSize - 1) / 2;
   }
   if (nPre > nPost) {
      if (nPre % nPost != 0 || !is_pow2(nPre / nPost)) return -1;
      return (patchSize - 1) * (nPre / nPost) / 2;
   }
   if (nPost % nPre != 0 || !is_pow2(nPost / nPre)) return -1;
   int ratio = nPost / nPre;
   if (patchSize % ratio != 0) return -1;
   return (patchSize / ratio) / 2;
}

/* components/PatchSize.cpp:98-130 */
int pvo_post_patch_size(int prePatchSize, int nPre, int nPost) {
   if (nPre == nPost) return prePatchSize;
   if (nPre > nPost) {
      if (nPre % nPost) return -1;
      return prePatchSize * (nPre / nPost);
   }
   if (nPost % nPre) return -1;
   int scale = nPost / nPre;
   if (prePatchSize % scale) return -1;
   return prePatchSize / scale;
}

/* PatchGeometry::verifyPatchSize (components/PatchGeometry.cpp:88-150), one axis. */
static int verify_axis(int nPre, int nPost, int patchSize) {
   if (nPre > nPost) {
      int s = nPre / nPost;
      return (s * nPost == nPre && is_pow2(s)) ? 0 : -1;
   }
   if (nPre < nPost) {
      int t = nPost / nPre;
      return (t * nPre == nPost && patchSize % t == 0 && is_pow2(t)) ? 0 : -1;
   }
   return (patchSize % 2 == 1) ? 0 : -1;
}

/* PatchGeometry::calcPatchStartInPost (components/PatchGeometry.cpp:334-390) */
static int patch_start_in_post(int indexRestrictedPre, int patchSize, int nPre, int nPost) {
   if (nPre == nPost) {
      return indexRestrictedPre - (patchSize - 1) / 2;
   }
   if (nPre < nPost) {
      int tstride = nPost / nPre;
      return indexRestrictedPre * tstride - (patchSize - tstride) / 2;
   }
   int stride = nPre / nPost;
   int extentOneSide = (stride / 2) * (patchSize - 1);
   float fStride = (float)stride;
   float fStart = (float)(indexRestrictedPre - extentOneSide);
   return (int)floorf(fStart / fStride);
}

/* PatchGeometry::calcPatchData (components/PatchGeometry.cpp:391-455) */
static void calc_patch_data(
      int index, int numPreRestricted, int preStartBorder, int numPostRestricted,
      int postStartBorder, int patchSize, int *patchDim, int *patchStart,
      int *postStartRes, int *postStartExt, int *postUnshrunkenStart) {
   int dim = patchSize, start = 0;
   int restrictedIndex = index - preStartBorder;
   int s = patch_start_in_post(restrictedIndex, patchSize, numPreRestricted, numPostRestricted);
   *postUnshrunkenStart = s + postStartBorder;
   int e = s + patchSize;
   if (e < 0) { int ex = -e; s += ex; e = 0; }
   if (s > numPostRestricted) { int ex = s - numPostRestricted; s = numPostRestricted; e -= ex; }
   if (s < 0) { int ex = -s; s = 0; dim -= ex; start = ex; }
   if (e > numPostRestricted) { int ex = e - numPostRestricted; e = numPostRestricted; dim -= ex; }
   if (dim < 0) dim = 0;
   *patchDim = dim;
   *patchStart = start;
   *postStartRes = s;
   *postStartExt = s + postStartBorder;
}

/* PatchGeometry::setPatchGeometry (components/PatchGeometry.cpp:179-262).
 * The x-axis pass hands calcPatchData the post halo's dn/up (not lt/rt), as the
 * reference does; the two agree whenever the halo is symmetric, which
 * LayerGeometry::requireMarginWidth guarantees. */
int pvo_patch_geometry(
      const pvo_loc *pre, const pvo_loc *post, int nxp, int nyp, pvo_patch *patches,
      int64_t *gSynPatchStart, int64_t *aPostOffset, int64_t *unshrunkenStart) {
   if (verify_axis(pre->nx, post->nx, nxp) || verify_axis(pre->ny, post->ny, nyp)) return -1;
   int npx = loc_nx_ext(pre), npy = loc_ny_ext(pre), npf = pre->nf;
   int *dimX = malloc(sizeof(int) * npx * 5), *dimY = malloc(sizeof(int) * npy * 5);
   if (!dimX || !dimY) { free(dimX); free(dimY); return -1; }
   int *startX = dimX + npx, *resX = dimX + 2 * npx, *extX = dimX + 3 * npx, *unsX = dimX + 4 * npx;
   int *startY = dimY + npy, *resY = dimY + 2 * npy, *extY = dimY + 3 * npy, *unsY = dimY + 4 * npy;
   for (int i = 0; i < npx; i++)
      calc_patch_data(i, pre->nx, pre->halo.lt, post->nx, post->halo.dn, nxp,
                      &dimX[i], &startX[i], &resX[i], &extX[i], &unsX[i]);
   for (int i = 0; i < npy; i++)
      calc_patch_data(i, pre->ny, pre->halo.dn, post->ny, post->halo.dn, nyp,
                      &dimY[i], &startY[i], &resY[i], &extY[i], &unsY[i]);
   int nxExtPost = loc_nx_ext(post), nyExtPost = loc_ny_ext(post);
   int numPatches = npx * npy * npf;
   for (int p = 0; p < numPatches; p++) {
      int xi = kxPos(p, npx, npy, npf), yi = kyPos(p, npx, npy, npf);
      if (patches) {
         patches[p].nx = (uint16_t)dimX[xi];
         patches[p].ny = (uint16_t)dimY[yi];
         patches[p].offset = (uint32_t)kIndex(startX[xi], startY[yi], 0, nxp, nyp, post->nf);
      }
      if (gSynPatchStart) gSynPatchStart[p] = kIndex(resX[xi], resY[yi], 0, post->nx, post->ny, post->nf);
      if (aPostOffset) aPostOffset[p] = kIndex(extX[xi], extY[yi], 0, nxExtPost, nyExtPost, post->nf);
      if (unshrunkenStart) unshrunkenStart[p] = kIndex(unsX[xi], unsY[yi], 0, nxExtPost, nyExtPost, post->nf);
   }
   free(dimX);
   free(dimY);
   return 0;
}

/* Weights::initNumDataPatches + calcDataIndexFromPatchIndex (components/Weights.cpp:178-232) */
int pvo_kernel_index_table(const pvo_loc *pre, const pvo_loc *post, int32_t *table) {
   int nkx = pre->nx > post->nx ? pre->nx / post->nx : 1;
   int nky = pre->ny > post->ny ? pre->ny / post->ny : 1;
   int nkf = pre->nf;
   if (table) {
      int npx = loc_nx_ext(pre), npy = loc_ny_ext(pre), npf = pre->nf;
      int numPatches = npx * npy * npf;
      for (int p = 0; p < numPatches; p++) {
         int x = (kxPos(p, npx, npy, npf) - pre->halo.lt) % nkx;
         if (x < 0) x += nkx;
         int y = (kyPos(p, npx, npy, npf) - pre->halo.up) % nky;
         if (y < 0) y += nky;
         table[p] = kIndex(x, y, featureIndex(p, npx, npy, npf), nkx, nky, nkf);
      }
   }
   return nkx * nky * nkf;
}

/* PatchGeometry::setTransposeItemIndices (components/PatchGeometry.cpp:264-332) and
 * TransposeWeights::transposeShared (utils/TransposeWeights.cpp:56-115). */
int pvo_transpose_shared(
      const pvo_loc *pre, const pvo_loc *post, int nxp, int nyp, const float *wPre, float *wPost) {
   if (verify_axis(pre->nx, post->nx, nxp) || verify_axis(pre->ny, post->ny, nyp)) return -1;
   int nfp = post->nf;
   int nkx = pre->nx > post->nx ? pre->nx / post->nx : 1;
   int nky = pre->ny > post->ny ? pre->ny / post->ny : 1;
   int nkf = pre->nf;
   int numKernels = nkx * nky * nkf;
   int patchSize = nxp * nyp * nfp;
   int xStride = pre->nx > post->nx ? pre->nx / post->nx : 1;
   int yStride = pre->ny > post->ny ? pre->ny / post->ny : 1;
   int xTStride = post->nx > pre->nx ? post->nx / pre->nx : 1;
   int yTStride = post->ny > pre->ny ? post->ny / pre->ny : 1;
   int nxpPost = nxp * xStride / xTStride;
   int nypPost = nyp * yStride / yTStride;
   /* post weights: geometry post->pre, kernels counted on the post layer */
   int nkxPost = post->nx > pre->nx ? post->nx / pre->nx : 1;
   int nkyPost = post->ny > pre->ny ? post->ny / pre->ny : 1;
   int nkfPost = post->nf;
   int patchSizePost = nxpPost * nypPost * pre->nf;
   for (int kp = 0; kp < numKernels; kp++) {
      for (int item = 0; item < patchSize; item++) {
         int kxPre = kxPos(kp, nkx, nky, nkf);
         int ixPre = kxPos(item, nxp, nyp, nfp);
         int ixConj = nxp - 1 - ixPre;
         int extX = (nxp - 1) * xStride / 2;
         int ksX = (kxPre - extX) % xStride;
         if (ksX < 0) ksX += xStride;
         int ixPost = (xStride * ixConj + ksX) / xTStride;
         int kyPre = kyPos(kp, nkx, nky, nkf);
         int iyPre = kyPos(item, nxp, nyp, nfp);
         int iyConj = nyp - 1 - iyPre;
         int extY = (nyp - 1) * yStride / 2;
         int ksY = (kyPre - extY) % yStride;
         if (ksY < 0) ksY += yStride;
         int iyPost = (yStride * iyConj + ksY) / yTStride;
         int ifPost = featureIndex(kp, nkx, nky, nkf);
         int itemPost = kIndex(ixPost, iyPost, ifPost, nxpPost, nypPost, nkf);

         int pxPost = 0;
         if (nkxPost > 1) {
            pxPost = (-(nxp - nkxPost) / 2 + ixPre) % nkxPost;
            if (pxPost < 0) pxPost += nkxPost;
         }
         int pyPost = 0;
         if (nkyPost > 1) {
            pyPost = (-(nyp - nkyPost) / 2 + iyPre) % nkyPost;
            if (pyPost < 0) pyPost += nkyPost;
         }
         int pfPost = featureIndex(item, nxp, nyp, nfp);
         int patchPost = kIndex(pxPost, pyPost, pfPost, nkxPost, nkyPost, nkfPost);
         wPost[(size_t)patchPost * patchSizePost + itemPost] = wPre[(size_t)kp * patchSize + item];
      }
   }
   return 0;
}

/* DataStore::updateActiveIndices (columns/DataStore.cpp:46-66) */
void pvo_compact(const float *aExt, int nbatch, int numExt, pvo_entry *entries, int64_t *numActive) {
   for (int b = 0; b < nbatch; b++) {
      const float *a = aExt + (size_t)b * numExt;
      pvo_entry *e = entries + (size_t)b * numExt;
      int64_t n = 0;
      for (int k = 0; k < numExt; k++) {
         if (a[k] != 0.0f) {
            e[n].index = (uint32_t)k;
            e[n].value = a[k];
            n++;
         }
      }
      numActive[b] = n;
   }
}

/* ANNActivityBuffer::setVertices / setSlopes (components/ANNActivityBuffer.cpp:227-400) */
int pvo_ann_vertices(
      float VThresh, float AMin, float AMax, float AShift, float VWidth,
      float *vV, float *vA, float *slopes) {
   if (VWidth < 0) { VThresh += VWidth; VWidth = -VWidth; }
   float V[4], A[4];
   int n;
   double slopeNeg, slopePos = 1.0;
   if (VThresh <= -(float)0.999 * FLT_MAX) {
      n = 1; V[0] = 0.0f; A[0] = -AShift; slopeNeg = 1.0;
   } else {
      if (VWidth == 0.0f && (float)VThresh - AShift == AMin) {
         n = 1; V[0] = VThresh; A[0] = AMin;
      } else {
         n = 2; V[0] = VThresh; V[1] = VThresh + VWidth; A[0] = AMin; A[1] = VThresh + VWidth - AShift;
      }
      slopeNeg = 0.0;
   }
   if (AMax < (float)0.999 * FLT_MAX) {
      if (A[n - 1] < AMax) {
         float interval = AMax - A[n - 1];
         V[n] = V[n - 1] + interval; A[n] = AMax; n++;
      } else {
         int v;
         for (v = n - 1; v >= 0; v--) if (A[v] < AMax) break;
         if (v >= 0) {
            float interval = AMax - A[v];
            n = v + 1;
            V[n] = V[v] + interval; A[n] = AMax; n++;
         } else {
            n = 1;
            if (slopeNeg > 0) {
               float iA = A[0] - AMax;
               float iV = (float)(iA / slopeNeg);
               V[0] = V[0] - iV; A[0] = AMax;
            } else {
               V[0] = 0.0f; A[0] = AMax; slopeNeg = 0;
            }
         }
      }
      slopePos = 0.0;
   }
   for (int i = 0; i < n; i++) { vV[i] = V[i]; vA[i] = A[i]; }
   slopes[0] = (float)slopeNeg;
   for (int k = 1; k < n; k++) {
      float v1 = V[k - 1], v2 = V[k];
      if (v1 != v2) slopes[k] = (A[k] - A[k - 1]) / (v2 - v1);
      else slopes[k] = A[k] > A[k - 1] ? INFINITY : (A[k] < A[k - 1] ? -INFINITY : NAN);
   }
   slopes[n] = (float)slopePos;
   return n;
}

/* AdaptiveTimeScaleController::calcTimesteps (components/AdaptiveTimeScaleController.cpp:57-86) */
void pvo_adaptive_timescale(
      int nbatch, double baseMax, double baseMin, double tauFactor, double growthFactor,
      const double *energies, double *st) {
   for (int b = 0; b < nbatch; b++) {
      double *s = st + 3 * b; /* timeScale, timeScaleMax, timeScaleTrue */
      double E0 = s[2];
      double Edt = energies[b];
      s[2] = Edt;
      if (Edt == E0) continue;
      double dE = (E0 - Edt) / s[0];
      if (dE < 0.0 || E0 <= 0.0 || Edt <= 0.0) {
         s[0] = baseMin;
         s[1] = baseMax;
      } else {
         double tauEff = E0 / dE;
         s[0] = tauFactor * tauEff;
         if (s[0] >= s[1]) {
            s[0] = s[1];
            s[1] *= (1 + growthFactor);
         }
      }
   }
}

/* ---------------- numeric loops, instantiated for float and double ---------------- */
#define REAL float
#define SUFFIX
#include "pvoracle_real.inc"
#undef REAL
#undef SUFFIX

#define REAL double
#define SUFFIX _f64
#include "pvoracle_real.inc"
#undef REAL
#undef SUFFIX

int pvo_deliver_pre_f64(
      const pvo_loc *pre, const pvo_loc *post, int nxp, int nyp, const double *w,
      const double *aExt, double dtFactor, double *gsyn) {
   return deliver_pre_dense_f64(pre, post, nxp, nyp, w, aExt, dtFactor, gsyn);
}

/* Sparse branch of PresynapticPerspectiveConvolveDelivery::deliver
 * (delivery/PresynapticPerspectiveConvolveDelivery.cpp:148-185): loop patch rows y, then the
 * active entries in list order, then the row's nk elements. */
static void deliver_pre_sparse_one(
      const pvo_loc *pre, const pvo_loc *post, int nxp, int nyp, const float *w,
      const pvo_patch *patches, const int64_t *gstart, const int32_t *ktab,
      const pvo_entry *ent, int64_t n, float dtFactor, float *g) {
   int nfp = post->nf;
   int sy = post->nx * post->nf;
   int syw = nxp * nfp;
   int patchSize = nxp * nyp * nfp;
   for (int y = 0; y < nyp; y++) {
      for (int64_t idx = 0; idx < n; idx++) {
         int k = (int)ent[idx].index;
         const pvo_patch *pt = &patches[k];
         if (y >= pt->ny) continue;
         float a = ent[idx].value;
         if (a == 0.0f) continue;
         a *= dtFactor;
         float *v = g + gstart[k] + (size_t)y * sy;
         const float *wv = w + (size_t)ktab[k] * patchSize + pt->offset + (size_t)y * syw;
         int nk = pt->nx * nfp;
         for (int i = 0; i < nk; i++) v[i] += a * wv[i];
      }
   }
}

int pvo_deliver_pre(
      const pvo_loc *pre, const pvo_loc *post, int nxp, int nyp, const float *w,
      const pvo_entry *entries, const int64_t *numActive, const float *aExt,
      float dtFactor, float *gsyn) {
   if (!entries) return deliver_pre_dense(pre, post, nxp, nyp, w, aExt, dtFactor, gsyn);
   int numPreExt = loc_num_ext(pre);
   pvo_patch *patches = malloc(sizeof(pvo_patch) * numPreExt);
   int64_t *gstart = malloc(sizeof(int64_t) * numPreExt);
   int32_t *ktab = malloc(sizeof(int32_t) * numPreExt);
   int rc = -1;
   if (patches && gstart && ktab &&
       pvo_patch_geometry(pre, post, nxp, nyp, patches, gstart, NULL, NULL) == 0) {
      pvo_kernel_index_table(pre, post, ktab);
      int numPostRes = loc_num_res(post);
      for (int b = 0; b < pre->nbatch; b++)
         deliver_pre_sparse_one(pre, post, nxp, nyp, w, patches, gstart, ktab,
                                entries + (size_t)b * numPreExt, numActive[b], dtFactor,
                                gsyn + (size_t)b * numPostRes);
      rc = 0;
   }
   free(patches);
   free(gstart);
   free(ktab);
   return rc;
}

/* GSynAccumulator.kpp:16-44: G = sum over channels of coeff[ch] * GSyn[ch], channel order. */
void pvo_gsyn_accumulate(int numNeuronsAcrossBatch, int numChannels, const float *coeffs, const float *gsyn, float *g) {
   for (int index = 0; index < numNeuronsAcrossBatch; index++) {
      float value = 0.0f;
      for (int ch = 0; ch < numChannels; ch++) value += coeffs[ch] * gsyn[(size_t)ch * numNeuronsAcrossBatch + index];
      g[index] = value;
   }
}

/* ---- LIF (components/LIFActivityComponent.cpp:332-942) ------------------------------------ */

/* Tausworthe generator of utils/cl_random.c (after GSL rng/taus.c): three shift-register
 * components; s0 holds the last output s1 ^ s2 ^ s3. */
static uint32_t taus_component(uint32_t s, int a, int b, uint32_t mask, int d) {
   return ((s & mask) << d) ^ (((s << a) ^ s) >> b);
}

static pvo_taus taus_next(pvo_taus t) {
   t.s1 = taus_component(t.s1, 13, 19, 4294967294u, 12);
   t.s2 = taus_component(t.s2, 2, 25, 4294967288u, 4);
   t.s3 = taus_component(t.s3, 3, 11, 4294967280u, 17);
   t.s0 = t.s1 ^ t.s2 ^ t.s3;
   return t;
}

/* cl_random_prob: the last output scaled to [0, 1) in float. */
static float taus_uniform(pvo_taus t) { return (float)t.s0 / 4294967296.0f; }

/* cl_random_init (utils/cl_random.c): element i is seeded with i + seed (0 counts as 1) through
 * three LCG steps, then warmed up by six generator steps; s0 = s1 ^ s2 ^ s3. */
void pvo_taus_init(pvo_taus *state, size_t count, uint32_t seed) {
   if (seed == 0) seed = 1;
   for (size_t i = 0; i < count; i++) {
      uint32_t s = (uint32_t)i + seed;
      if (s == 0) s = 1;
      pvo_taus t;
      t.s1 = 69069u * s;
      t.s2 = 69069u * t.s1;
      t.s3 = 69069u * t.s2;
      for (int w = 0; w < 6; w++) t = taus_next(t);
      t.s0 = t.s1 ^ t.s2 ^ t.s3;
      state[i] = t;
   }
}

void pvo_taus_next(pvo_taus *state, size_t count) {
   for (size_t i = 0; i < count; i++) state[i] = taus_next(state[i]);
}

/* Noise on one conductance input: one draw decides whether an event happens this step (rate
 * freq in Hz over dt in seconds), a second draw scales its amplitude. */
static float lif_noise(pvo_taus *r, float gsyn, float dtSec, float freq, float amp) {
   *r = taus_next(*r);
   if (taus_uniform(*r) < dtSec * freq) {
      *r = taus_next(*r);
      gsyn = gsyn + amp * taus_uniform(*r);
   }
   return gsyn;
}

/* dV/dt of the conductance-based membrane (LIF_Vmem_derivative). */
static float lif_dvdt(float v, float ge, float gi, float gib, const pvo_lif_params *p) {
   float g = 1.0f + ge + gi + gib;
   float vinf = (p->Vrest + p->Vexc * ge + p->Vinh * gi + p->VinhB * gib) / g;
   return g * (vinf - v) / p->tau;
}

/* One LIF timestep for every restricted neuron (index k across the batch), in the reference's
 * float arithmetic: noise on the three GSyn channels (EXC, INH, INHB at channel offsets
 * c * nbatch * numNeurons), the conductance and membrane update of the method ('a' arma filter,
 * 'b' Heun with conductances at both ends of the step, 'o' exponential Euler with end-of-step
 * conductances), the threshold relaxation, and the spike (A = 1 at the extended index, V reset to
 * Vrest, Vth += deltaVth, G_IB += deltaGIB).  GMAX = 10 caps each conductance. */
int pvo_lif_update(char method, const pvo_loc *loc, const pvo_lif_params *p, float dt, pvo_taus *rnd, float *V,
                   float *Vth, float *GE, float *GI, float *GIB, const float *gsynHead, float *aExt) {
   if (method != 'a' && method != 'b' && method != 'o') return -1;
   const float GMAX = 10.0f;
   const int numNeurons = loc_num_res(loc);
   const int numExt = loc_num_ext(loc);
   const int total = numNeurons * loc->nbatch;
   const float eE = expf(-dt / p->tauE), eI = expf(-dt / p->tauI), eIB = expf(-dt / p->tauIB);
   const float eVth = expf(-dt / p->tauVth);
   const float dtSec = 0.001f * dt;
   const float *gsE = gsynHead, *gsI = gsynHead + total, *gsIB = gsynHead + 2 * (size_t)total;
   for (int k = 0; k < total; k++) {
      const int b = k / numNeurons, kr = k % numNeurons;
      const int kex = b * numExt + kIndexExtended(kr, loc->nx, loc->ny, loc->nf, loc->halo.lt, loc->halo.rt,
                                                  loc->halo.dn, loc->halo.up);
      pvo_taus r = rnd[k];
      float v = V[k], vth = Vth[k], ge = GE[k], gi = GI[k], gib = GIB[k];
      float inE = lif_noise(&r, gsE[k], dtSec, p->noiseFreqE, p->noiseAmpE);
      float inI = lif_noise(&r, gsI[k], dtSec, p->noiseFreqI, p->noiseAmpI);
      float inIB = lif_noise(&r, gsIB[k], dtSec, p->noiseFreqIB, p->noiseAmpIB);
      if (method == 'o') {
         ge = inE + ge * eE;
         gi = inI + gi * eI;
         gib = inIB + gib * eIB;
         ge = ge > GMAX ? GMAX : ge;
         gi = gi > GMAX ? GMAX : gi;
         gib = gib > GMAX ? GMAX : gib;
         float tauInf = (dt / p->tau) * (1.0f + ge + gi + gib);
         float vInf = (p->Vrest + ge * p->Vexc + gi * p->Vinh + gib * p->VinhB) / (1.0f + ge + gi + gib);
         v = vInf + (v - vInf) * expf(-tauInf);
      } else {
         float ge0 = ge + inE, gi0 = gi + inI, gib0 = gib + inIB;
         float tauInf0 = 0.0f, vInf0 = 0.0f;
         if (method == 'a') {  /* before the cap */
            tauInf0 = p->tau / (1 + ge0 + gi0 + gib0);
            vInf0 = (p->Vrest + p->Vexc * ge0 + p->Vinh * gi0 + p->VinhB * gib0) / (1 + ge0 + gi0 + gib0);
         }
         ge0 = ge0 > GMAX ? GMAX : ge0;
         gi0 = gi0 > GMAX ? GMAX : gi0;
         gib0 = gib0 > GMAX ? GMAX : gib0;
         float ge1 = ge0 * eE, gi1 = gi0 * eI, gib1 = gib0 * eIB;
         if (method == 'b') {
            float d1 = lif_dvdt(v, ge0, gi0, gib0, p);
            float d2 = lif_dvdt(v + dt * d1, ge1, gi1, gib1, p);
            float d = (d1 + d2) * 0.5f;
            v = v + dt * d;
         } else {
            /* the end-of-step time constant takes the start-of-step G_IB, as the reference does */
            float tauInf1 = p->tau / (1 + ge1 + gi1 + gib0);
            float vInf1 = (p->Vrest + p->Vexc * ge1 + p->Vinh * gi1 + p->VinhB * gib1) / (1 + ge1 + gi1 + gib1);
            float slope = (tauInf1 - tauInf0) / dt;
            float f1 = slope == 0.0f ? expf(-dt / tauInf0) : powf(tauInf1 / tauInf0, -1 / slope);
            float f2 = slope == -1.0f ? tauInf0 / dt * logf(tauInf1 / tauInf0 + 1.0f)
                                      : (1 - tauInf0 / dt * (1 - f1)) / (1 + slope);
            float f3 = 1.0f - f1 - f2;
            v = f1 * v + f2 * vInf0 + f3 * vInf1;
         }
         ge = ge1;
         gi = gi1;
         gib = gib1;
      }
      vth = p->VthRest + (vth - p->VthRest) * eVth;
      const int fired = v > vth;
      aExt[kex] = fired ? 1.0f : 0.0f;
      if (fired) {
         v = p->Vrest;
         vth = vth + p->deltaVth;
         gib = gib + p->deltaGIB;
      }
      rnd[k] = r;
      V[k] = v;
      Vth[k] = vth;
      GE[k] = ge;
      GI[k] = gi;
      GIB[k] = gib;
   }
   return 0;
}

/* ---- MomentumUpdater (weightupdaters/MomentumUpdater.cpp:291-345) ---------------------------- */

/* The momentum factors of applyMomentum: viscosity dwFactor = exp(-1/tau) (0 when tau is 0),
 * simple and alex dwFactor = tau; wFactor = momentumDecay, times dWMax for alex. */
int pvo_momentum_factors(char method, float tau, float decay, float dWMax, float *dwFactor, float *wFactor) {
   switch (method) {
      case 'v': *dwFactor = tau != 0.0f ? expf(-1.0f / tau) : 0.0f; *wFactor = decay; return 0;
      case 's': *dwFactor = tau; *wFactor = decay; return 0;
      case 'a': *dwFactor = tau; *wFactor = decay * dWMax; return 0;
      default: return -1;
   }
}

/* applyMomentum, then prev_dW = dW and HebbianUpdater::updateWeights (W += dW), element by
 * element in float: dW = dW * (1 - f); dW = dW + f * prev; dW = dW - g * W. */
void pvo_momentum_update_weights(int64_t n, float dwFactor, float wFactor, float *dw, float *prevDw, float *w) {
   const float keep = 1 - dwFactor;
   for (int64_t k = 0; k < n; k++) {
      float d = dw[k] * keep;
      d = d + dwFactor * prevDw[k];
      d = d - wFactor * w[k];
      dw[k] = d;
      prevDw[k] = d;
      w[k] = w[k] + d;
   }
}
