// Stand-in for OpenPV's utils/PVLog.hpp: Fatal() / FatalIf record the message and throw, so that
// the test harness can report a refusal instead of ending the process.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdarg>
#include <cstdio>
#include <stdexcept>
#include <string>
namespace PVStandin {
struct FatalError : std::runtime_error {
   using std::runtime_error::runtime_error;
};
struct FatalStream {
   [[noreturn]] void printf(char const *fmt, ...) {
      char buf[1024];
      va_list ap;
      va_start(ap, fmt);
      std::vsnprintf(buf, sizeof buf, fmt, ap);
      va_end(ap);
      throw FatalError(buf);
   }
};
} // namespace PVStandin
#define Fatal(...) ::PVStandin::FatalStream()
#define FatalIf(cond, ...)                            \
   do {                                               \
      if (cond) ::PVStandin::FatalStream().printf(__VA_ARGS__); \
   } while (0)
#define pvAssert(c) ((void)0)
