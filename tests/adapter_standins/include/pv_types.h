// Stand-in for OpenPV's include/pv_types.h: channel codes and the activity cube.  TEST
// INFRASTRUCTURE ONLY.
#ifndef PV_TYPES_H_
#define PV_TYPES_H_
#include "PVLayerLoc.h"
enum ChannelType {
   CHANNEL_EXC      = 0,
   CHANNEL_INH      = 1,
   CHANNEL_INHB     = 2,
   CHANNEL_GAP      = 3,
   CHANNEL_NORM     = 4,
   CHANNEL_NOUPDATE = -1
};
typedef struct PVLayerCube_ {
   int numItems;
   float const *data;
   PVLayerLoc loc;
   int isSparse;
   long const *numActive;
   void const *activeIndices;
} PVLayerCube;
#endif
