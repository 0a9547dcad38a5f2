// ref_delivery_shim.cpp -- C entry points that run the reference's own CPU delivery loops
// (PresynapticPerspectiveConvolveDelivery::deliver and PostsynapticPerspectiveConvolveDelivery::deliver,
// compiled from the reference tree with the stand-ins in oracle/refshim), single-threaded.
// TEST INFRASTRUCTURE ONLY (oracle/_ref).
#include "PostsynapticPerspectiveConvolveDelivery.hpp"
#include "PresynapticPerspectiveConvolveDelivery.hpp"

#include <cstdint>
#include <cstring>
#include <exception>
#include <vector>

extern "C" {

struct pvr_loc2 {
   int nbatch, nx, ny, nf;
   int lt, rt, dn, up;
};

static PVLayerLoc to_loc2(pvr_loc2 const *l) {
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

// Presynaptic delivery: entries (SparseList<float>::Entry per batch element, stride numPreExt) or
// dense aExt when entries is NULL.  gsyn is accumulated into.
int pvr_deliver_pre(pvr_loc2 const *pre, pvr_loc2 const *post, int nxp, int nyp, float const *w, void const *entries,
                    int64_t const *numActive, float const *aExt, float *gsyn) {
   try {
      PVLayerLoc preLoc = to_loc2(pre), postLoc = to_loc2(post);
      PV::Weights weights(preLoc, postLoc, nxp, nyp, w);
      PV::WeightsPair wp;
      wp.pre = &weights;
      PV::ArborList arbors;
      PV::PreData preData;
      preData.loc = preLoc;
      preData.sparse = entries != nullptr;
      std::vector<long> num(pre->nbatch, 0);
      int numExt = (pre->nx + pre->lt + pre->rt) * (pre->ny + pre->dn + pre->up) * pre->nf;
      std::vector<float> zeros;
      PVLayerCube &cube = preData.publisher.cube;
      std::memset(&cube, 0, sizeof(cube));
      cube.loc = preLoc;
      cube.numItems = numExt * pre->nbatch;
      if (entries) {
         for (int b = 0; b < pre->nbatch; b++) num[b] = (long)numActive[b];
         zeros.assign((size_t)numExt * pre->nbatch, 0.0f);
         cube.data = zeros.data();
         cube.isSparse = 1;
         cube.numActive = num.data();
         cube.activeIndices = entries;
      } else {
         cube.data = aExt;
      }
      PV::PostGSyn postGSyn;
      postGSyn.loc = postLoc;
      PV::PresynapticPerspectiveConvolveDelivery d;
      d.wire(&preData, &postGSyn, &wp, &arbors);
      d.deliver(gsyn);
   } catch (std::exception const &) {
      return -1;
   }
   return 0;
}

// Postsynaptic delivery from src (activity aExt) into tgt; wPost are the post-perspective weights
// (kernels of the tgt->src geometry, patch nxpPost x nypPost x src.nf).
int pvr_deliver_post(pvr_loc2 const *src, pvr_loc2 const *tgt, int nxpPost, int nypPost, float const *wPost,
                     float const *aExt, float *gsyn) {
   try {
      PVLayerLoc srcLoc = to_loc2(src), tgtLoc = to_loc2(tgt);
      PV::Weights postWeights(tgtLoc, srcLoc, nxpPost, nypPost, wPost);
      PV::WeightsPair wp;
      wp.post = &postWeights;
      PV::ArborList arbors;
      PV::PreData preData;
      preData.loc = srcLoc;
      PVLayerCube &cube = preData.publisher.cube;
      std::memset(&cube, 0, sizeof(cube));
      cube.loc = srcLoc;
      cube.data = aExt;
      cube.numItems = (src->nx + src->lt + src->rt) * (src->ny + src->dn + src->up) * src->nf * src->nbatch;
      PV::PostGSyn postGSyn;
      postGSyn.loc = tgtLoc;
      PV::PostsynapticPerspectiveConvolveDelivery d;
      d.wire(&preData, &postGSyn, &wp, &arbors);
      d.deliver(gsyn);
   } catch (std::exception const &) {
      return -1;
   }
   return 0;
}

}  // extern "C"
