// Stand-in for OpenPV's include/PVLayerLoc.h (same structs and field order), so that the
// adapters compile without the reference tree.  TEST INFRASTRUCTURE ONLY.
#ifndef PVLAYERLOC_H_
#define PVLAYERLOC_H_
typedef struct PVHalo_ {
   int lt, rt, dn, up;
} PVHalo;
typedef struct PVLayerLoc_ {
   int nbatch, nx, ny, nf;
   int nbatchGlobal, nxGlobal, nyGlobal;
   int kb0, kx0, ky0;
   PVHalo halo;
} PVLayerLoc;
#endif
