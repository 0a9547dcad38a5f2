// Stand-in for OpenPV's structures/Patch.hpp.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdint>
namespace PV {
struct Patch {
   std::uint16_t nx, ny;
   std::uint32_t offset;
};
} // namespace PV
