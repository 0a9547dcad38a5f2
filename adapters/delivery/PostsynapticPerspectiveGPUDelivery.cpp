// PostsynapticPerspectiveGPUDelivery.cpp -- replacement body of the reference's translation unit
// of the same name (delivery/PostsynapticPerspectiveGPUDelivery.cpp), for the class its
// unchanged header declares (delivery/PostsynapticPerspectiveGPUDelivery.hpp).  The framework
// side (device buffers requested, the copy of a stale datastore, the arbor loop) is the
// reference's contract; the delivery is libpvgpu in place of CudaRecvPost, whose cuDNN
// convolution needed three permute kernels and a separate output buffer
// (cudakernels/CudaRecvPost.cpp:357-389, arch/cuda/CudaKernel.cu:20-135):
//   * pvgpu_deliver_post_tc -- the tcgen05 tensor-core implicit GEMM (split-TF32 operands, FP32
//     within 1e-5 of the FP32 sums) -- where the shape fits (one-to-one connections with feature
//     counts that are multiples of 32);
//   * pvgpu_deliver_post -- the FP32 kernel -- everywhere else.
// Both read the datastore in OpenPV's own layout and accumulate into the channel's GSyn.  The
// member the header reserves for the cuDNN path's output buffer (mCudnnGSyn) holds the
// tensor-core entry's weight workspace; mRecvKernel and mDevicePostToPreActivity stay empty.
// Non-shared weights are refused at allocation (Fatal).
#include "delivery/PostsynapticPerspectiveGPUDelivery.hpp"
#include "pvgpu_adapter.hpp"
#include "utils/conversions.hpp"

namespace PV {

PostsynapticPerspectiveGPUDelivery::PostsynapticPerspectiveGPUDelivery(
      char const *name,
      PVParams *params,
      Communicator const *comm) {
   mCorrectReceiveGpu = true;
   initialize(name, params, comm);
}

PostsynapticPerspectiveGPUDelivery::PostsynapticPerspectiveGPUDelivery() { mCorrectReceiveGpu = true; }

PostsynapticPerspectiveGPUDelivery::~PostsynapticPerspectiveGPUDelivery() {
   delete mRecvKernel;
   delete mDevicePostToPreActivity;
   delete mCudnnGSyn;
}

void PostsynapticPerspectiveGPUDelivery::initialize(
      char const *name,
      PVParams *params,
      Communicator const *comm) {
   mReceiveGpu = true; // this class is the receiveGpu = true, postsynaptic, convolve delivery
   BaseObject::initialize(name, params, comm);
}

void PostsynapticPerspectiveGPUDelivery::setObjectType() {
   mObjectType = "PostsynapticPerspectiveGPUDelivery";
}

// The connection as the library describes it: pre -> post with the presynaptic-perspective
// patch size; the weights it reads are the postsynaptic-perspective ones.
static pvgpu_conn_desc connectionOf(
      PVLayerLoc const *preLoc,
      PVLayerLoc const *postLoc,
      Weights const *preWeights,
      float dtFactor) {
   pvgpu_conn_desc conn;
   conn.pre       = PVGpuAdapter::toLoc(preLoc);
   conn.post      = PVGpuAdapter::toLoc(postLoc);
   conn.nxp       = preWeights->getPatchSizeX();
   conn.nyp       = preWeights->getPatchSizeY();
   conn.dt_factor = dtFactor;
   return conn;
}

Response::Status PostsynapticPerspectiveGPUDelivery::communicateInitInfo(
      std::shared_ptr<CommunicateInitInfoMessage const> message) {
   auto status = HyPerDelivery::communicateInitInfo(message);
   if (!Response::completed(status) or getChannelCode() == CHANNEL_NOUPDATE) {
      return status;
   }
   // the library reads the dense presynaptic datastore and the postsynaptic-perspective
   // weights on the device, and accumulates into the device GSyn
   mWeightsPair->needPost();
   mPreData->setAllocCudaDatastore();
   mWeightsPair->getPostWeights()->useGPU();
   mPostGSyn->useCuda();
   return Response::SUCCESS;
}

Response::Status
PostsynapticPerspectiveGPUDelivery::setCudaDevice(std::shared_ptr<SetCudaDeviceMessage const> message) {
   auto status = HyPerDelivery::setCudaDevice(message);
   if (status != Response::SUCCESS or getChannelCode() == CHANNEL_NOUPDATE) {
      return status;
   }
   mWeightsPair->getPostWeights()->setCudaDevice(message->mCudaDevice);
   mCudaDevice = message->mCudaDevice;
   return status;
}

Response::Status PostsynapticPerspectiveGPUDelivery::allocateDataStructures() {
   FatalIf(
         mCudaDevice == nullptr,
         "%s received AllocateData without having received SetCudaDevice.\n",
         getDescription_c());
   if (mWeightsPair and !mWeightsPair->getDataStructuresAllocatedFlag()) {
      return Response::POSTPONE;
   }
   if (mPostGSyn and !mPostGSyn->getDataStructuresAllocatedFlag()) {
      return Response::POSTPONE;
   }
   auto status = HyPerDelivery::allocateDataStructures();
   if (!Response::completed(status) or getChannelCode() == CHANNEL_NOUPDATE) {
      return status;
   }
   FatalIf(
         !mWeightsPair->getPostWeights()->getSharedFlag(),
         "%s: libpvgpu delivers shared weights only (sharedWeights = false is not supported).\n",
         getDescription_c());
   pvgpu_conn_desc const conn = connectionOf(
         mPreData->getLayerLoc(), mPostGSyn->getLayerLoc(), mWeightsPair->getPreWeights(), mDeltaTimeFactor);
   std::size_t const workspaceBytes = pvgpu_deliver_tc_workspace_bytes(&conn);
   if (workspaceBytes > 0) {
      mCudnnGSyn = mCudaDevice->createBuffer(workspaceBytes, &getDescription());
   }
   return Response::SUCCESS;
}

Response::Status PostsynapticPerspectiveGPUDelivery::copyInitialStateToGPU() {
   initializeRecvKernelArgs();
   return Response::SUCCESS;
}

// Nothing is staged ahead of the first delivery; what is checked here is what the library
// would refuse.
void PostsynapticPerspectiveGPUDelivery::initializeRecvKernelArgs() {
   if (getChannelCode() == CHANNEL_NOUPDATE) {
      return;
   }
   FatalIf(
         mPreData->getCudaDatastore() == nullptr or mPostGSyn->getCudaBuffer() == nullptr
               or mWeightsPair->getPostWeights()->getDeviceData() == nullptr,
         "%s: device buffers missing after allocation.\n",
         getDescription_c());
}

void PostsynapticPerspectiveGPUDelivery::deliver(float *destBuffer) {
   if (getChannelCode() == CHANNEL_NOUPDATE) {
      return;
   }
   (void)destBuffer; // the GPU deliveries accumulate into the device copy of the channel
   Weights *postWeights       = mWeightsPair->getPostWeights();
   pvgpu_conn_desc const conn = connectionOf(
         mPreData->getLayerLoc(), mPostGSyn->getLayerLoc(), mWeightsPair->getPreWeights(), mDeltaTimeFactor);
   float *gsyn = static_cast<float *>(mPostGSyn->getCudaBuffer()->getPointer())
                 + (std::size_t)getChannelCode() * (std::size_t)mPostGSyn->getBufferSizeAcrossBatch();
   std::size_t const arborSize =
         (std::size_t)postWeights->getNumDataPatches() * (std::size_t)postWeights->getPatchSizeOverall();
   float const *weightsDevice = static_cast<float const *>(postWeights->getDeviceData()->getPointer());
   cudaStream_t stream        = mCudaDevice->getStream();

   int const numArbors = mArborList->getNumAxonalArbors();
   for (int arbor = 0; arbor < numArbors; arbor++) {
      if (mPreData->getUpdatedCudaDatastoreFlag()) {
         PVLayerCube const cube = mPreData->getPublisher()->createCube(mArborList->getDelay(arbor));
         mPreData->getCudaDatastore()->copyToDevice(cube.data);
         mPreData->setUpdatedCudaDatastoreFlag(false);
      }
      float const *aExt = static_cast<float const *>(mPreData->getCudaDatastore()->getPointer());
      float const *w    = weightsDevice + (std::size_t)arbor * arborSize;
      pvgpu_status status = PVGPU_ERR_UNSUPPORTED_SHAPE;
      if (mCudnnGSyn) {
         status = pvgpu_deliver_post_tc(
               &conn, aExt, w, gsyn, mCudnnGSyn->getPointer(), mCudnnGSyn->getSize(), stream);
      }
      if (status == PVGPU_ERR_UNSUPPORTED_SHAPE) {
         status = pvgpu_deliver_post(&conn, aExt, w, gsyn, PVGPU_DELIVER_FAST, stream);
      }
      PVGpuAdapter::check(status, "pvgpu_deliver_post", getDescription_c());
   }
}

// The unit-input response on the host, as in the reference: for every restricted postsynaptic
// neuron the sum of its receptive field's weights, row by row, times dt_factor.
void PostsynapticPerspectiveGPUDelivery::deliverUnitInput(float *recvBuffer) {
   if (getChannelCode() == CHANNEL_NOUPDATE) {
      return;
   }
   PVLayerLoc const *loc = mPostGSyn->getLayerLoc();
   int const numPostRes  = mPostGSyn->getBufferSize();
   Weights *postWeights  = mWeightsPair->getPostWeights();
   int const syp         = postWeights->getPatchStrideY();
   int const rowLength   = postWeights->getPatchSizeX() * postWeights->getPatchSizeF();
   int const numArbors   = mArborList->getNumAxonalArbors();
   for (int arbor = 0; arbor < numArbors; arbor++) {
      for (int b = 0; b < loc->nbatch; b++) {
         float *recv = recvBuffer + (std::size_t)b * numPostRes;
         for (int ky = 0; ky < postWeights->getPatchSizeY(); ky++) {
            for (int k = 0; k < numPostRes; k++) {
               int const kExt = kIndexExtended(
                     k, loc->nx, loc->ny, loc->nf, loc->halo.lt, loc->halo.rt, loc->halo.dn, loc->halo.up);
               float const *w = postWeights->getDataFromPatchIndex(arbor, kExt) + ky * syp;
               float sum      = 0.0f;
               for (int i = 0; i < rowLength; i++) {
                  sum += w[i];
               }
               recv[k] += mDeltaTimeFactor * sum;
            }
         }
      }
   }
}

} // end namespace PV
