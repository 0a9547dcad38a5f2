// HyPerLCAInternalStateBuffer.cu -- replacement of the reference's GPU translation unit of the
// same name (components/HyPerLCAInternalStateBuffer.cu): runKernel() calls libpvgpu's LCA update
// (pvgpu_lca_update, the counterpart of updateHyPerLCAOnGPU, HyPerLCAInternalStateBuffer.kpp:18-63,
// with the same arguments) on the device buffers the component already owns.  Products and
// sums are rounded as the reference's CPU path rounds them, so the GPU run reproduces the CPU
// path's V.
#include "components/HyPerLCAInternalStateBuffer.hpp"
#include "pvgpu_adapter.hpp"

namespace PV {

void HyPerLCAInternalStateBuffer::runKernel() {
   pvgpu_loc const loc = PVGpuAdapter::toLoc(getLayerLoc());
   PVGpuAdapter::check(
         pvgpu_lca_update(
               &loc,
               mSelfInteract ? 1 : 0,
               static_cast<double const *>(mCudaDtAdapt->getPointer()),
               (float)mScaledTimeConstantTau,
               static_cast<float const *>(mAccumulatedGSyn->getCudaBuffer()->getPointer()),
               static_cast<float const *>(mActivity->getCudaBuffer()->getPointer()),
               static_cast<float *>(getCudaBuffer()->getPointer()),
               mCudaDevice->getStream()),
         "pvgpu_lca_update",
         getDescription_c());
}

} // end namespace PV
