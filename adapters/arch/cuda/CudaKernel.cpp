// CudaKernel.cpp -- the launcher base class declared by adapters/arch/cuda/CudaKernel.hpp, in
// place of the reference's arch/cuda/CudaKernel.cpp (which defines the cuDNN error helper and
// so needs <cudnn.h>).  Launch shapes: the grid is the global work size divided by the local
// work size, rounded up, per dimension; shapes beyond the device's limits end the run (Fatal),
// as launch errors do after do_run().  The six-argument run() takes (x, y, f) work sizes and
// launches f on the grid's x dimension, x on y and y on z, as the reference's does.
#include "arch/cuda/CudaKernel.hpp"
#include "arch/cuda/cuda_util.hpp"
#include "utils/PVAssert.hpp"
#include "utils/PVLog.hpp"

namespace PVCuda {

CudaKernel::CudaKernel(CudaDevice *inDevice)
      : device(inDevice), argsSet(false), dimsSet(false), mKernelName(nullptr) {}

CudaKernel::CudaKernel() : CudaKernel(nullptr) {}

CudaKernel::~CudaKernel() {}

int CudaKernel::run() {
   int const result = do_run();
   handleCallError(mKernelName);
   return result;
}

int CudaKernel::run(long global_work_size) { return run(global_work_size, 1L); }

int CudaKernel::run(long global_work_size, long local_work_size) {
   setDims(global_work_size, 1, 1, local_work_size, 1, 1);
   return run();
}

int CudaKernel::run_nocheck(long global_work_size, long local_work_size) {
   setDims(global_work_size, 1, 1, local_work_size, 1, 1, false);
   return run();
}

int CudaKernel::run(long gWorkSizeX, long gWorkSizeY, long lWorkSizeX, long lWorkSizeY) {
   setDims(gWorkSizeX, gWorkSizeY, 1, lWorkSizeX, lWorkSizeY, 1);
   return run();
}

int CudaKernel::run_nocheck(long gWorkSizeX, long gWorkSizeY, long lWorkSizeX, long lWorkSizeY) {
   setDims(gWorkSizeX, gWorkSizeY, 1, lWorkSizeX, lWorkSizeY, 1, false);
   return run();
}

int CudaKernel::run(
      long gWorkSizeX,
      long gWorkSizeY,
      long gWorkSizeF,
      long lWorkSizeX,
      long lWorkSizeY,
      long lWorkSizeF) {
   setDims(gWorkSizeF, gWorkSizeX, gWorkSizeY, lWorkSizeF, lWorkSizeX, lWorkSizeY);
   return run();
}

void CudaKernel::setDims(
      long gWorkSizeX,
      long gWorkSizeY,
      long gWorkSizeF,
      long lWorkSizeX,
      long lWorkSizeY,
      long lWorkSizeF,
      bool error) {
   FatalIf(device == nullptr, "CudaKernel %s: no device.\n", mKernelName ? mKernelName : "");
   long const global[3] = {gWorkSizeX, gWorkSizeY, gWorkSizeF};
   long const local[3]  = {lWorkSizeX, lWorkSizeY, lWorkSizeF};
   long grid[3];
   long threads = 1;
   for (int d = 0; d < 3; d++) {
      FatalIf(local[d] <= 0 or global[d] < 0, "CudaKernel: work size %ld / %ld in dimension %d.\n", global[d], local[d], d);
      if (error) {
         pvAssert(global[d] % local[d] == 0);
      }
      grid[d] = (global[d] + local[d] - 1) / local[d];
      FatalIf(
            grid[d] > device->get_max_grid_size_dimension(d),
            "CudaKernel: %ld blocks in dimension %d exceed the device's %d.\n",
            grid[d],
            d,
            device->get_max_grid_size_dimension(d));
      FatalIf(
            local[d] > device->get_max_block_size_dimension(d),
            "CudaKernel: %ld threads in dimension %d exceed the device's %d.\n",
            local[d],
            d,
            device->get_max_block_size_dimension(d));
      threads *= local[d];
   }
   FatalIf(
         threads > device->get_max_threads(),
         "CudaKernel: %ld threads per block exceed the device's %d.\n",
         threads,
         device->get_max_threads());
   grid_size  = dim3((unsigned)grid[0], (unsigned)grid[1], (unsigned)grid[2]);
   block_size = dim3((unsigned)local[0], (unsigned)local[1], (unsigned)local[2]);
   dimsSet    = true;
}

} // namespace PVCuda
