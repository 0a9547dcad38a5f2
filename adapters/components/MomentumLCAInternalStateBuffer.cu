// MomentumLCAInternalStateBuffer.cu -- replacement of the reference's GPU translation unit of the
// same name (components/MomentumLCAInternalStateBuffer.cu): runKernel() calls libpvgpu's momentum
// LCA update (pvgpu_momentum_lca_update, the counterpart of updateMomentumLCAOnGPU,
// MomentumLCAInternalStateBuffer.kpp:18-69, with the same arguments) on the device buffers the
// component already owns: V, the previous drive, the accumulated GSyn and the activity.
#include "components/MomentumLCAInternalStateBuffer.hpp"
#include "pvgpu_adapter.hpp"

namespace PV {

void MomentumLCAInternalStateBuffer::runKernel() {
   pvgpu_loc const loc = PVGpuAdapter::toLoc(getLayerLoc());
   PVGpuAdapter::check(
         pvgpu_momentum_lca_update(
               &loc,
               mSelfInteract ? 1 : 0,
               mLCAMomentumRate,
               static_cast<double const *>(mCudaDtAdapt->getPointer()),
               (float)mScaledTimeConstantTau,
               static_cast<float const *>(mAccumulatedGSyn->getCudaBuffer()->getPointer()),
               static_cast<float const *>(mActivity->getCudaBuffer()->getPointer()),
               static_cast<float *>(mPrevDrive->getCudaBuffer()->getPointer()),
               static_cast<float *>(getCudaBuffer()->getPointer()),
               mCudaDevice->getStream()),
         "pvgpu_momentum_lca_update",
         getDescription_c());
}

} // end namespace PV
