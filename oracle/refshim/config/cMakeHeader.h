/* cMakeHeader.h -- build configuration for compiling reference CPU sources in oracle/_ref:
 * every optional feature of src/cMakeHeader.template off (no MPI, no OpenMP threads, no CUDA,
 * no cuDNN, no Lua), i.e. the reference's single-process, single-thread CPU build.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef CMAKEHEADER_H_
#define CMAKEHEADER_H_
#endif
