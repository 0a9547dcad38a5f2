// GSynAccumulator.cu -- replacement of the reference's GPU translation unit of the same name
// (components/GSynAccumulator.cu): runKernel() calls libpvgpu's channel accumulation
// (pvgpu_gsyn_accumulate, the counterpart of updateGSynAccumulatorOnGPU, GSynAccumulator.kpp:16-44)
// on the component's device buffers.  The library takes the channel coefficients from the host
// array the component keeps (mChannelCoefficients); the device copy the reference kernel read
// (mCudaChannelCoefficients) is left unused.
#include "components/GSynAccumulator.hpp"
#include "pvgpu_adapter.hpp"

namespace PV {

void GSynAccumulator::runKernel() {
   PVLayerLoc const *loc = getLayerLoc();
   int64_t const numNeuronsAcrossBatch = (int64_t)loc->nx * loc->ny * loc->nf * loc->nbatch;
   PVGpuAdapter::check(
         pvgpu_gsyn_accumulate(
               numNeuronsAcrossBatch,
               mNumInputChannels,
               mChannelCoefficients.data(),
               static_cast<float const *>(mLayerInput->getCudaBuffer()->getPointer()),
               static_cast<float *>(getCudaBuffer()->getPointer()),
               mCudaDevice->getStream()),
         "pvgpu_gsyn_accumulate",
         getDescription_c());
}

} // end namespace PV
