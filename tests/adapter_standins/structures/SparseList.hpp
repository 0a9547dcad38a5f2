// Stand-in for OpenPV's structures/SparseList.hpp: the entry layout only.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdint>
namespace PV {
template <typename T>
class SparseList {
  public:
   struct Entry {
      uint32_t index;
      T value;
   };
};
} // namespace PV
