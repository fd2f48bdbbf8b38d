// Host-side checks exported by libsubsweep_gpu.so beside the C ABI: the runtime's own
// timestep scheduling (TimestepState in sweep_host.cpp), callable without a device so
// the CPU tests can hold it against the reference's known answers
// (src/sweep/timestep_state.rs:98-137), and the checkpoint validation of
// sw_load_state.  Not part of the drop-in interface.
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The levels of one step's sweeps in order after `advances` calls of
 * advance_allowed_levels, for `num_levels` levels (1..16).  Writes at most `cap`
 * entries; returns the number of sweeps, or -1 on an invalid argument. */
int32_t sw_host_sweep_order(int32_t num_levels, int32_t advances, int32_t* out, int32_t cap);

/* The lowest allowed level after `advances` calls; -1 on an invalid argument. */
int32_t sw_host_lowest_allowed(int32_t num_levels, int32_t advances);

/* The validation sw_load_state applies to a checkpoint buffer before anything reaches
 * the device: the header's magic, version and timestep state, the buffer's length,
 * and every cell's timestep level below the header's level count.  Returns 0 for a
 * buffer that passes, 1 for a bad header, 2 for a short buffer, 3 for a level out of
 * range. */
int32_t sw_host_check_checkpoint(const void* buffer, size_t bytes);

/* The schedule positions sw_create lays out for one task space from the tasks' Kahn
 * levels (task_level[t] for t = dir * np + cell, levels 0..levels-1; cells >= n are
 * padding): the d directions cut into `groups` contiguous groups, each group's tasks
 * after the previous group's, by level, in task-id order within a level.  Writes
 * order[n * d] and the segment offsets seg[0..segments] (at most seg_cap entries);
 * returns the number of segments, -1 on an invalid argument. */
int64_t sw_host_schedule_order(const uint16_t* task_level, uint32_t np, uint32_t n, uint32_t d, int32_t levels,
                               int32_t groups, uint32_t* order, uint32_t* seg, int64_t seg_cap);

/* Task spaces of fewer than 2^31 tasks that sw_create splits the mixed path's
 * directions into at the least (0: more than eight would be needed); -1 on an invalid
 * argument. */
int32_t sw_host_task_spaces(uint32_t np, int32_t d);

/* Direction groups of the schedule for d directions, `tasks` tasks and `levels` Kahn
 * levels (SUBSWEEP_DIR_GROUPS overrides); -1 on an invalid argument. */
int32_t sw_host_dir_groups(int32_t d, uint64_t tasks, int64_t levels);

#ifdef __cplusplus
}
#endif
