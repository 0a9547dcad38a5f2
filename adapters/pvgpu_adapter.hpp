// pvgpu_adapter.hpp -- shared by the replacement translation units under adapters/: OpenPV
// layer locations to the C ABI's, and OpenPV's error convention on top of the ABI's status
// codes.  OpenPV treats every CUDA error as fatal (handleError, arch/cuda/cuda_util.hpp:14-27);
// the adapters keep that behaviour: a call of libpvgpu that does not return PVGPU_OK ends the
// run through Fatal() with the library's status and message.
#ifndef PVGPU_ADAPTER_HPP_
#define PVGPU_ADAPTER_HPP_

#include "include/PVLayerLoc.h"
#include "pvgpu.h"
#include "structures/SparseList.hpp"
#include "utils/PVLog.hpp"

// The active-index lists the framework keeps on the device are passed to the library as they
// are: one SparseList<float>::Entry is one pvgpu_entry.
static_assert(sizeof(PV::SparseList<float>::Entry) == sizeof(pvgpu_entry), "SparseList entry layout");
static_assert(sizeof(long) == sizeof(int64_t), "numActive is long in OpenPV, int64_t in the library");

namespace PVGpuAdapter {

inline pvgpu_loc toLoc(PVLayerLoc const *l) {
   pvgpu_loc r;
   r.nbatch  = l->nbatch;
   r.nx      = l->nx;
   r.ny      = l->ny;
   r.nf      = l->nf;
   r.halo.lt = l->halo.lt;
   r.halo.rt = l->halo.rt;
   r.halo.dn = l->halo.dn;
   r.halo.up = l->halo.up;
   return r;
}

inline void check(pvgpu_status status, char const *call, char const *owner) {
   if (status != PVGPU_OK) {
      Fatal().printf(
            "%s: %s failed: %s (%s)\n", owner, call, pvgpu_status_string(status), pvgpu_last_error());
   }
}

} // namespace PVGpuAdapter

#endif // PVGPU_ADAPTER_HPP_
