// ISTAInternalStateBuffer.cu -- replacement of the reference's GPU translation unit of the same
// name (components/ISTAInternalStateBuffer.cu): runKernel() calls libpvgpu's ISTA update
// (pvgpu_ista_update, the counterpart of updateISTAInternalStateBufferOnGPU,
// ISTAInternalStateBuffer.kpp:16-63, with the same arguments) on the device buffers the component
// already owns.
#include "components/ISTAInternalStateBuffer.hpp"
#include "pvgpu_adapter.hpp"

namespace PV {

void ISTAInternalStateBuffer::runKernel() {
   pvgpu_loc const loc = PVGpuAdapter::toLoc(getLayerLoc());
   PVGpuAdapter::check(
         pvgpu_ista_update(
               &loc,
               mActivity->getVThresh(),
               static_cast<double const *>(mCudaDtAdapt->getPointer()),
               mScaledTimeConstantTau,
               static_cast<float const *>(mAccumulatedGSyn->getCudaBuffer()->getPointer()),
               static_cast<float const *>(mActivity->getCudaBuffer()->getPointer()),
               static_cast<float *>(getCudaBuffer()->getPointer()),
               mCudaDevice->getStream()),
         "pvgpu_ista_update",
         getDescription_c());
}

} // end namespace PV
