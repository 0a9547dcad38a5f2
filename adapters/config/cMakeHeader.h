/* cMakeHeader.h -- the build configuration the adapters are compiled against (the reference
 * generates this file from src/cMakeHeader.template): the CUDA build with OpenMP threads, no
 * cuDNN (libpvgpu replaces the cuDNN delivery), no MPI, no Lua. */
#ifndef CMAKEHEADER_H_
#define CMAKEHEADER_H_
#define PV_VERSION_MAJOR 3
#define PV_VERSION_MINOR 0
#define PV_DIR "."
#define PV_USE_OPENMP_THREADS
#define PV_USE_CUDA
#endif
