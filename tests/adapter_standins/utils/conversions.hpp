// Stand-in for OpenPV's utils/conversions.hpp: the restricted -> extended index.  TEST
// INFRASTRUCTURE ONLY.
#pragma once
inline int kIndexExtended(int k, int nx, int ny, int nf, int lt, int rt, int dn, int up) {
   (void)ny;
   (void)dn;
   int const f = k % nf, x = (k / nf) % nx, y = k / (nf * nx);
   return ((y + up) * (nx + lt + rt) + (x + lt)) * nf + f;
}
