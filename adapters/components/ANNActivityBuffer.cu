// ANNActivityBuffer.cu -- replacement of the reference's GPU translation unit of the same name
// (components/ANNActivityBuffer.cu): runKernel() calls libpvgpu's vertex-form transfer function
// (pvgpu_ann_vertices, the counterpart of applyVerticesANNActivityBufferOnGPU,
// ANNActivityBuffer.kpp:16-77) with the vertex arrays the component keeps on the device, so
// vertex lists given in params work as well as the ones derived from VThresh / AMin / AMax /
// AShift / VWidth.
#include "components/ANNActivityBuffer.hpp"
#include "pvgpu_adapter.hpp"

namespace PV {

void ANNActivityBuffer::runKernel() {
   pvgpu_loc const loc = PVGpuAdapter::toLoc(getLayerLoc());
   PVGpuAdapter::check(
         pvgpu_ann_vertices(
               &loc,
               mNumVertices,
               static_cast<float const *>(mCudaVerticesV->getPointer()),
               static_cast<float const *>(mCudaVerticesA->getPointer()),
               static_cast<float const *>(mCudaSlopes->getPointer()),
               static_cast<float const *>(mInternalState->getCudaBuffer()->getPointer()),
               static_cast<float *>(getCudaBuffer()->getPointer()),
               mCudaDevice->getStream()),
         "pvgpu_ann_vertices",
         getDescription_c());
}

} // end namespace PV
