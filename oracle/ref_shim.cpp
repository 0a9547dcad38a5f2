// ref_shim.cpp -- C entry points around OpenPV reference code compiled from the
// reference source tree (TEST INFRASTRUCTURE ONLY; built by oracle/Makefile.ref
// into oracle/_ref/libpvref.so, never shipped).
//
// Compiled from the reference, unmodified, where they lie:
//   components/PatchGeometry.cpp            (PV::PatchGeometry)
//   components/HyPerLCAInternalStateBuffer.kpp  (PV::updateHyPerLCAOnCPU)
//   components/MomentumLCAInternalStateBuffer.kpp  (PV::updateMomentumLCAOnCPU)
//   components/ISTAInternalStateBuffer.kpp  (PV::updateISTAInternalStateBufferOnCPU)
//   components/GSynAccumulator.kpp          (PV::updateGSynAccumulatorOnCPU)
//   components/ANNActivityBuffer.kpp        (PV::applyVerticesANNActivityBufferOnCPU)
//   probes/CostFunctions.hpp                (L2/L1/firm-threshold cost functions)
// plus utils/{PVLog,PathComponents,PVAssert,ExpandLeadingTilde}.cpp that they link against.
// These checks pin the oracle's geometry and update restatements bit for bit.

#include "components/PatchGeometry.hpp"
#include "components/HyPerLCAInternalStateBuffer.kpp"
#include "components/ISTAInternalStateBuffer.kpp"
#include "components/MomentumLCAInternalStateBuffer.kpp"
#include "components/GSynAccumulator.kpp"
#include "components/ANNActivityBuffer.kpp"
#include "probes/CostFunctions.hpp"

#include <cstdint>
#include <cstring>
#include <exception>

extern "C" {

struct pvr_loc {
   int nbatch, nx, ny, nf;
   int lt, rt, dn, up;
};

static PVLayerLoc to_loc(pvr_loc const *l) {
   PVLayerLoc loc;
   std::memset(&loc, 0, sizeof(loc));
   loc.nbatch = l->nbatch;
   loc.nx = l->nx;
   loc.ny = l->ny;
   loc.nf = l->nf;
   loc.nbatchGlobal = l->nbatch;
   loc.nxGlobal = l->nx;
   loc.nyGlobal = l->ny;
   loc.halo.lt = l->lt;
   loc.halo.rt = l->rt;
   loc.halo.dn = l->dn;
   loc.halo.up = l->up;
   return loc;
}

// PatchGeometry tables for a pre->post connection.  Returns 0, or -1 when the reference
// rejects the geometry (it throws std::runtime_error from verifyPatchSize).
int pvr_patch_geometry(
      pvr_loc const *pre, pvr_loc const *post, int nxp, int nyp, uint16_t *patchNx, uint16_t *patchNy,
      uint32_t *patchOffset, int64_t *gSynPatchStart, int64_t *aPostOffset, int64_t *unshrunkenStart,
      int32_t *transposeItemIndex) {
   PVLayerLoc preLoc = to_loc(pre), postLoc = to_loc(post);
   try {
      PV::PatchGeometry g("ref", nxp, nyp, postLoc.nf, &preLoc, &postLoc);
      g.allocateDataStructures();
      int n = g.getNumPatches();
      for (int p = 0; p < n; p++) {
         PV::Patch const &pt = g.getPatch(p);
         patchNx[p] = pt.nx;
         patchNy[p] = pt.ny;
         patchOffset[p] = pt.offset;
         gSynPatchStart[p] = (int64_t)g.getGSynPatchStart(p);
         aPostOffset[p] = (int64_t)g.getAPostOffset(p);
         unshrunkenStart[p] = (int64_t)g.getUnshrunkenStart(p);
      }
      if (transposeItemIndex) {
         int nk = g.getNumKernels(), ps = g.getPatchSizeOverall();
         for (int k = 0; k < nk; k++)
            for (int i = 0; i < ps; i++) transposeItemIndex[(size_t)k * ps + i] = g.getTransposeItemIndex(k, i);
      }
   } catch (std::exception const &) {
      return -1;
   }
   return 0;
}

void pvr_lca_update(
      pvr_loc const *l, int selfInteract, double const *dtAdapt, float tau, float const *g, float const *aExt,
      float *v) {
   PV::updateHyPerLCAOnCPU(l->nbatch, l->nx * l->ny * l->nf, l->nx, l->ny, l->nf, l->lt, l->rt, l->dn, l->up,
                           selfInteract != 0, dtAdapt, tau, g, aExt, v);
}

void pvr_momentum_lca_update(
      pvr_loc const *l, int selfInteract, float momentumRate, double const *dtAdapt, float tau, float const *g,
      float const *aExt, float *prevDrive, float *v) {
   PV::updateMomentumLCAOnCPU(l->nbatch, l->nx * l->ny * l->nf, l->nx, l->ny, l->nf, l->lt, l->rt, l->dn, l->up,
                              selfInteract != 0, momentumRate, dtAdapt, tau, g, aExt, prevDrive, v);
}

void pvr_ista_update(
      pvr_loc const *l, float VThresh, double const *dtAdapt, float tau, float const *g, float const *aExt, float *v) {
   PV::updateISTAInternalStateBufferOnCPU(l->nbatch, l->nx * l->ny * l->nf, l->nx, l->ny, l->nf, l->lt, l->rt, l->dn,
                                          l->up, VThresh, dtAdapt, tau, g, aExt, v);
}

void pvr_gsyn_accumulate(int n, int numChannels, float const *coeffs, float const *gsyn, float *out) {
   PV::updateGSynAccumulatorOnCPU(n, numChannels, coeffs, gsyn, out);
}

void pvr_apply_vertices(
      pvr_loc const *l, int numVertices, float const *vV, float const *vA, float const *slopes, float const *v,
      float *aExt) {
   PV::applyVerticesANNActivityBufferOnCPU(l->nbatch, l->nx * l->ny * l->nf, l->nx, l->ny, l->nf, l->lt, l->rt,
                                           l->dn, l->up, numVertices, vV, vA, slopes, v, aExt);
}

// kind: 0 = L2, 1 = L1, 2 = firm threshold (p0 = VThresh, p1 = VWidth); value-wise cost.
double pvr_cost(int kind, double p0, double p1, double x) {
   if (kind == 0) return PV::L2CostFunction()(x);
   if (kind == 1) return PV::L1CostFunction()(x);
   return PV::FirmThresholdCostFunction(p0, p1)(x);
}

} // extern "C"
