// PresynapticPerspectiveGPUDelivery.cpp -- replacement body of the reference's translation unit
// of the same name (delivery/PresynapticPerspectiveGPUDelivery.cpp), for the class its
// unchanged header declares (delivery/PresynapticPerspectiveGPUDelivery.hpp).  The framework
// side -- which buffers the delivery asks its layers to keep on the device, the host->device
// copy of a stale datastore, the arbor / delay loop -- is the reference's contract; the
// delivery itself is one call of libpvgpu per arbor in place of CudaRecvPre (a global-atomic
// scatter, cudakernels/CudaRecvPre.cu:10-88): pvgpu_deliver_pre reads the SparseList (or the
// dense datastore) and accumulates into the channel's GSyn with no atomics.
//
// Differences from the reference GPU path, all on purpose:
//   * the patch tables it copied to the device (mDevicePatches, mDeviceGSynPatchStart) are not
//     needed -- the library derives each patch from the layer geometry -- and are not made;
//   * each arbor reads its own weights (arbor offset into the device weights); the reference
//     kernel read arbor 0's for every arbor;
//   * dt_factor multiplies each contribution once (the reference's dense GPU path applied it
//     twice, CudaRecvPre.cu:42,84; it is 1 for convolve deliveries);
//   * non-shared weights are refused at allocation (Fatal): the library handles shared weights.
#include "delivery/PresynapticPerspectiveGPUDelivery.hpp"
#include "pvgpu_adapter.hpp"

namespace PV {

PresynapticPerspectiveGPUDelivery::PresynapticPerspectiveGPUDelivery(
      char const *name,
      PVParams *params,
      Communicator const *comm) {
   mCorrectReceiveGpu = true;
   initialize(name, params, comm);
}

PresynapticPerspectiveGPUDelivery::PresynapticPerspectiveGPUDelivery() { mCorrectReceiveGpu = true; }

PresynapticPerspectiveGPUDelivery::~PresynapticPerspectiveGPUDelivery() {}

void PresynapticPerspectiveGPUDelivery::initialize(
      char const *name,
      PVParams *params,
      Communicator const *comm) {
   mReceiveGpu = true; // this class is the receiveGpu = true, presynaptic, convolve delivery
   BaseObject::initialize(name, params, comm);
}

void PresynapticPerspectiveGPUDelivery::setObjectType() {
   mObjectType = "PresynapticPerspectiveGPUDelivery";
}

Response::Status PresynapticPerspectiveGPUDelivery::communicateInitInfo(
      std::shared_ptr<CommunicateInitInfoMessage const> message) {
   auto status = HyPerDelivery::communicateInitInfo(message);
   if (!Response::completed(status) or getChannelCode() == CHANNEL_NOUPDATE) {
      return status;
   }
   // The library reads the presynaptic datastore (and, for a sparse layer, its SparseList) and
   // the presynaptic-perspective weights on the device, and accumulates into the device GSyn.
   mWeightsPair->needPre();
   mPreData->setAllocCudaDatastore();
   if (mPreData->getSparseLayer()) {
      mPreData->setAllocCudaActiveIndices();
   }
   mWeightsPair->getPreWeights()->useGPU();
   mPostGSyn->useCuda();
   return status;
}

Response::Status
PresynapticPerspectiveGPUDelivery::setCudaDevice(std::shared_ptr<SetCudaDeviceMessage const> message) {
   auto status = HyPerDelivery::setCudaDevice(message);
   if (status != Response::SUCCESS or getChannelCode() == CHANNEL_NOUPDATE) {
      return status;
   }
   mWeightsPair->getPreWeights()->setCudaDevice(message->mCudaDevice);
   mCudaDevice = message->mCudaDevice;
   return status;
}

Response::Status PresynapticPerspectiveGPUDelivery::allocateDataStructures() {
   FatalIf(
         mCudaDevice == nullptr,
         "%s received AllocateData without having received SetCudaDevice.\n",
         getDescription_c());
   if (mWeightsPair and !mWeightsPair->getDataStructuresAllocatedFlag()) {
      return Response::POSTPONE;
   }
   auto status = HyPerDelivery::allocateDataStructures();
   if (!Response::completed(status) or getChannelCode() == CHANNEL_NOUPDATE) {
      return status;
   }
   FatalIf(
         !mWeightsPair->getPreWeights()->getSharedFlag(),
         "%s: libpvgpu delivers shared weights only (sharedWeights = false is not supported).\n",
         getDescription_c());
   return Response::SUCCESS;
}

Response::Status PresynapticPerspectiveGPUDelivery::copyInitialStateToGPU() {
   initializeRecvKernelArgs();
   return Response::SUCCESS;
}

// Nothing is staged ahead of the first delivery: the library takes the layer geometry and the
// device pointers at each call.  What is checked here is what the library would refuse.
void PresynapticPerspectiveGPUDelivery::initializeRecvKernelArgs() {
   if (getChannelCode() == CHANNEL_NOUPDATE) {
      return;
   }
   PVLayerLoc const *preLoc = mPreData->getLayerLoc();
   FatalIf(
         preLoc->halo.lt != preLoc->halo.rt or preLoc->halo.dn != preLoc->halo.up,
         "%s: libpvgpu needs equal left/right and up/down margins on the presynaptic layer.\n",
         getDescription_c());
   FatalIf(
         mPreData->getCudaDatastore() == nullptr or mPostGSyn->getCudaBuffer() == nullptr
               or mWeightsPair->getPreWeights()->getDeviceData() == nullptr,
         "%s: device buffers missing after allocation.\n",
         getDescription_c());
}

void PresynapticPerspectiveGPUDelivery::deliver(float *destBuffer) {
   if (getChannelCode() == CHANNEL_NOUPDATE) {
      return;
   }
   (void)destBuffer; // the GPU deliveries accumulate into the device copy of the channel
   Weights *weights = mWeightsPair->getPreWeights();
   pvgpu_conn_desc conn;
   conn.pre       = PVGpuAdapter::toLoc(mPreData->getLayerLoc());
   conn.post      = PVGpuAdapter::toLoc(mPostGSyn->getLayerLoc());
   conn.nxp       = weights->getPatchSizeX();
   conn.nyp       = weights->getPatchSizeY();
   conn.dt_factor = mDeltaTimeFactor;
   float *gsyn    = static_cast<float *>(mPostGSyn->getCudaBuffer()->getPointer())
                 + (std::size_t)getChannelCode() * (std::size_t)mPostGSyn->getBufferSizeAcrossBatch();
   std::size_t const arborSize =
         (std::size_t)weights->getNumDataPatches() * (std::size_t)weights->getPatchSizeOverall();
   float const *weightsDevice = static_cast<float const *>(weights->getDeviceData()->getPointer());
   bool const sparse          = mPreData->getSparseLayer();
   cudaStream_t stream        = mCudaDevice->getStream();

   int const numArbors = mArborList->getNumAxonalArbors();
   for (int arbor = 0; arbor < numArbors; arbor++) {
      // a datastore the host has written since the last device copy goes to the device first
      if (mPreData->getUpdatedCudaDatastoreFlag()) {
         PVLayerCube const cube = mPreData->getPublisher()->createCube(mArborList->getDelay(arbor));
         mPreData->getCudaDatastore()->copyToDevice(cube.data);
         if (cube.isSparse) {
            mPreData->getCudaNumActive()->copyToDevice(cube.numActive);
            mPreData->getCudaActiveIndices()->copyToDevice(cube.activeIndices);
         }
         mPreData->setUpdatedCudaDatastoreFlag(false);
      }
      auto const *entries = sparse ? static_cast<pvgpu_entry const *>(mPreData->getCudaActiveIndices()->getPointer())
                                   : nullptr;
      auto const *numActive =
            sparse ? static_cast<int64_t const *>(mPreData->getCudaNumActive()->getPointer()) : nullptr;
      auto const *aExt =
            sparse ? nullptr : static_cast<float const *>(mPreData->getCudaDatastore()->getPointer());
      PVGpuAdapter::check(
            pvgpu_deliver_pre(
                  &conn,
                  entries,
                  numActive,
                  aExt,
                  weightsDevice + (std::size_t)arbor * arborSize,
                  gsyn,
                  PVGPU_DELIVER_FAST,
                  stream),
            "pvgpu_deliver_pre",
            getDescription_c());
   }
}

// The unit-input response (every presynaptic neuron at activity 1), on the host as in the
// reference: each patch row y of every presynaptic neuron's shrunken patch adds its weights
// times dt_factor into the host buffer, row-major over y then presynaptic index -- the
// reference's single-thread order.
void PresynapticPerspectiveGPUDelivery::deliverUnitInput(float *recvBuffer) {
   PVLayerLoc const *preLoc  = mPreData->getLayerLoc();
   PVLayerLoc const *postLoc = mPostGSyn->getLayerLoc();
   int const numPreExt = (preLoc->nx + preLoc->halo.lt + preLoc->halo.rt)
                         * (preLoc->ny + preLoc->halo.dn + preLoc->halo.up) * preLoc->nf;
   int const numPostRes = postLoc->nx * postLoc->ny * postLoc->nf;
   int const sy         = postLoc->nx * postLoc->nf;
   Weights *weights     = mWeightsPair->getPreWeights();
   int const syw        = weights->getPatchStrideY();
   int const nfp        = weights->getPatchSizeF();
   auto const &gSynPatchStart = weights->getGeometry()->getGSynPatchStart();
   int const numArbors        = mArborList->getNumAxonalArbors();
   for (int arbor = 0; arbor < numArbors; arbor++) {
      for (int b = 0; b < postLoc->nbatch; b++) {
         float *recv = recvBuffer + (std::size_t)b * numPostRes;
         for (int y = 0; y < weights->getPatchSizeY(); y++) {
            for (int k = 0; k < numPreExt; k++) {
               Patch const &patch = weights->getPatch(k);
               if (y >= patch.ny) {
                  continue;
               }
               float const *w = weights->getDataFromPatchIndex(arbor, k) + patch.offset + y * syw;
               float *g       = recv + gSynPatchStart[k] + y * sy;
               int const n    = patch.nx * nfp;
               for (int i = 0; i < n; i++) {
                  g[i] += mDeltaTimeFactor * w[i];
               }
            }
         }
      }
   }
}

} // end namespace PV
