// database_constants.h -- the parameter header the reference reads
// (src/includes/database_constants.h), for the dump build only.  It keeps the
// reference's names and meanings, because the reference's sources include it
// by that name, and selects a database small enough to dump and to replay on
// the CPU:
//   default       PolyDegree 2048, CoeffMods {60, 60}: the active preset's
//                 parameters (database_constants.h:215-223) with 4096 entries
//                 (256 x 16, the oracle's smallest case)
//   PIN_N4096     PolyDegree 4096, CoeffMods {60, 60, 60}: the "2^14 * 24KB"
//                 preset's parameters (database_constants.h:92-101) with 1024
//                 entries (256 x 4)
// The build script puts this directory ahead of src/includes on the include
// path; the reference's own sources stay untouched.
#pragma once
#include <array>
#include <cstddef>

namespace DatabaseConstants {
#ifdef PIN_N4096
constexpr size_t MaxFstDimSz = 256;
constexpr size_t PolyDegree = 4096;
constexpr size_t NumEntries = 1024;
constexpr size_t EntrySize = 0;
constexpr size_t GSW_L = 4;
constexpr size_t GSW_L_KEY = 8;
constexpr size_t PlainMod = 46;
constexpr size_t SmallQWidth = 57;
constexpr std::array<size_t, 3> CoeffMods = {60, 60, 60};
#else
constexpr size_t MaxFstDimSz = 256;
constexpr size_t PolyDegree = 2048;
constexpr size_t NumEntries = 4096;
constexpr size_t EntrySize = 0;
constexpr size_t GSW_L = 5;
constexpr size_t GSW_L_KEY = 10;
constexpr size_t PlainMod = 16;
constexpr size_t SmallQWidth = 27;
constexpr std::array<size_t, 2> CoeffMods = {60, 60};
#endif
}  // namespace DatabaseConstants
