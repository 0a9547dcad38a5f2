// CudaKernel.hpp -- stands in for the reference's arch/cuda/CudaKernel.hpp in a build whose GPU
// deliveries are libpvgpu's.  The reference header includes <cudnn.h> unconditionally (line 12)
// for one static helper (cudnnHandleError), which ties every CUDA build to cuDNN even when
// PV_USE_CUDNN is off.  This header declares the same kernel-launcher base class without that
// helper and without the cuDNN permute launchers, so nothing in the build includes cuDNN.  It
// keeps the reference header's include guard: whichever of the two is reached first is the one
// used, and the declarations a translation unit sees are the same apart from the cuDNN parts.
// Placed ahead of the reference tree on the include path (adapters/ first).
#ifndef CUDAKERNEL_HPP_
#define CUDAKERNEL_HPP_

#include "arch/cuda/CudaDevice.hpp"
#include <cstdlib>

namespace PVCuda {

// Base of the framework's CUDA kernels: a subclass sets its arguments, then one of the run()
// overloads sets the launch shape from global / local work sizes and calls do_run().
class CudaKernel {
  public:
   CudaKernel(CudaDevice *inDevice);
   CudaKernel();
   virtual ~CudaKernel();

   int run(); // the subclass picks its own launch shape
   int run(long global_work_size);
   int run(long global_work_size, long local_work_size);
   int run_nocheck(long global_work_size, long local_work_size);
   int run(long gWorkSizeX, long gWorkSizeY, long lWorkSizeX, long lWorkSizeY);
   int run_nocheck(long gWorkSizeX, long gWorkSizeY, long lWorkSizeX, long lWorkSizeY);
   int
   run(long gWorkSizeX,
       long gWorkSizeY,
       long gWorkSizeF,
       long lWorkSizeX,
       long lWorkSizeY,
       long lWorkSizeF);

  protected:
   virtual int do_run() = 0;

   void setArgsFlag() { argsSet = true; }

   dim3 grid_size;
   dim3 block_size;
   CudaDevice *device;
   bool argsSet;
   bool dimsSet;
   char const *mKernelName;

  private:
   void setDims(
         long gWorkSizeX,
         long gWorkSizeY,
         long gWorkSizeF,
         long lWorkSizeX,
         long lWorkSizeY,
         long lWorkSizeF,
         bool error = true);
};

} // namespace PVCuda

#endif // CUDAKERNEL_HPP_
