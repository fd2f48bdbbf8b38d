// Types and constants shared by the host runtime and the sweep kernels.
#pragma once

#include <cstdint>

namespace swk {

// Face geometry in FP64: normal and area in one 32-byte load.
struct alignas(32) Geo64 {
  double x, y, z, w;
};

constexpr int kMaxFaces = 64;       // per cell (validated at upload)
constexpr int kMaxDirections = 128;
constexpr uint32_t kKindShift = 30;
constexpr uint32_t kNbrMask = (1u << kKindShift) - 1;
constexpr uint32_t kKindLocal = 0, kKindPeriodic = 1, kKindBoundary = 2;
constexpr uint32_t kEmptySlot = 0xffffffffu;
// stable compaction of schedule positions (pull path): threads per block, positions per
// thread, positions per chunk
constexpr int kCompactThreads = 256;
constexpr int kCompactPer = 8;
constexpr uint32_t kCompactChunk = kCompactThreads * kCompactPer;

enum : uint32_t { kErrStall = 1u, kErrQueue = 2u, kErrClamp = 8u, kErrRecords = 16u };

// Control block of one handle (device memory).
struct SweepCtl {
  unsigned long long head;  // next ready-queue slot to claim (consumers); pull wavefront: barrier arrivals
  unsigned long long tail;  // next ready-queue slot to fill (producers)
  uint32_t error;           // kErr* bits
  uint32_t pad;
  unsigned long long tasks;     // solved tasks (cumulative)
  unsigned long long chem_cells;
  unsigned long long chem_attempts;
  unsigned long long chem_failures;
  unsigned long long attempts;  // task attempts of the pull transport (retries included)
  uint32_t n_ge[32];       // number of cells with level >= l (current level assignment)
  uint32_t hist[32];       // scratch level histogram
  // scalars of a step replayed from a CUDA graph, copied in by the graph's first node
  uint32_t epoch_base;     // sweep number before the step's first sweep
  uint32_t pad2;
  double time;             // simulation time at the end of the step
};

}  // namespace swk
