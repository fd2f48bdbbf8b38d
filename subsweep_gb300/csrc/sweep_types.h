// Types and constants shared by the host runtime and the sweep kernels.
#pragma once

#include <cstdint>

namespace swk {

// Face geometry in FP64: normal and area in one 32-byte load.
struct alignas(32) Geo64 {
  double x, y, z, w;
};

constexpr int kMaxFaces = 64;       // per cell (validated at upload)
constexpr int kMaxDirWords = 4;     // <= 128 directions
constexpr int kWarpsPerBlock = 8;
constexpr uint32_t kKindShift = 30;
constexpr uint32_t kNbrMask = (1u << kKindShift) - 1;
constexpr uint32_t kKindLocal = 0, kKindPeriodic = 1, kKindBoundary = 2;

enum : uint32_t { kErrStall = 1u, kErrRounds = 2u, kErrFrontier = 4u, kErrClamp = 8u };

// Control block of one handle (device memory).
struct SweepCtl {
  uint32_t count[3];       // frontier sizes, rotating by round (see k_sweep)
  uint32_t bar_count;      // grid barrier arrivals
  uint32_t bar_gen;        // grid barrier generation
  uint32_t error;          // kErr* bits
  uint32_t rounds;         // rounds of the last sweep
  uint32_t pad;
  unsigned long long tasks;     // solved tasks (cumulative)
  unsigned long long visits;    // cell visits (cumulative)
  unsigned long long chem_cells;
  unsigned long long chem_attempts;
  unsigned long long chem_failures;
  uint32_t n_ge[32];       // number of cells with level >= l (current level assignment)
  uint32_t hist[32];       // scratch histogram for level sorting
  uint32_t fill[32];       // scratch offsets for level sorting
};

}  // namespace swk
