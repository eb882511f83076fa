// Host-side launchers shared by the translation units of libdiffvg_gb300.
#pragma once

#include <cuda_runtime.h>

#include "dvg_device.cuh"

namespace dvg {

// Error reporting shared by the C ABI entry points (a thread-local fixed
// buffer returned by dvg_last_error; printf-style, allocation-free).
int fail(int status, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
void clear_error();
// Host-side checks of a scene description; writes the first point of every
// path segment to seg_point when it is not NULL.
int validate_desc(const DvgSceneDesc *d, int *seg_point);
int count_stroke_records(const DvgSceneDesc *d);

// Scene preparation from the parameter arena: transforms, boxes, segment
// order, boundary CDFs and the per-tile candidate group lists.
// tile_cap is the capacity of S.tile_list; bin_total receives the list
// length.  On overflow the lists are emptied and DVG_EFLAG_BIN_OVERFLOW is
// raised in S.err.
cudaError_t launch_prepare(const DevScene &S, int tile_cap, int *bin_total, int4 *g_tile_range, int *tile_count,
                           cudaStream_t st);

// One launcher per render kernel; the C ABI sequences them (and can record
// CUDA events between them for per-kernel timing).
void launch_weight(const DevScene &S, const DevRender &R, cudaStream_t st);
void launch_sample_fwd(const DevScene &S, const DevRender &R, float4 *samples, cudaStream_t st,
                       const EdgeRecords *deferral = nullptr);
void launch_hit_check(const float *params, const float *fwd_params, int n, unsigned *stale, cudaStream_t st);
void launch_resolve(const DevRender &R, const float4 *samples, float *image, cudaStream_t st);
// dbg_val / dbg_flag: per-sample background adjoint scratch (only written
// when R.d_background is set).
void launch_sample_bwd(const DevScene &S, const DevRender &R, float4 *dbg_val, int *dbg_flag, cudaStream_t st);
void launch_bg_combine(const DevScene &S, const DevRender &R, const float4 *dbg_val, const int *dbg_flag,
                       cudaStream_t st);
void launch_edge(const DevScene &S, const DevRender &R, const EdgeRecords &E, cudaStream_t st);
// launch_edge in two halves: drawing and ordering the boundary samples, then
// evaluating them (the batched path evaluates every scene's in one launch)
void launch_edge_setup(const DevScene &S, const DevRender &R, const EdgeRecords &E, cudaStream_t st);
void launch_edge_eval(const DevScene &S, const DevRender &R, const EdgeRecords &E, cudaStream_t st);
// Persistent batched passes over nb scenes B[order[r]] (device arrays);
// item_start[r] is the first work item of the r-th scene (nb + 1 entries),
// spt the 32-sample chunks per item, counter a device int (zeroed here).
// The boundary pass takes the scenes with paired lanes (8+ groups) only;
// wide: every scene's walks take the wide queues (DevScene::wide_queues).
void launch_batch_sample_fwd(const BatchScene *B, int nb, const int *order, const int *item_start, int spt,
                             int ctas_per_sm, int *counter, bool wide, cudaStream_t st);
void launch_batch_sample_bwd(const BatchScene *B, int nb, const int *order, const int *item_start, int spt,
                             int ctas_per_sm, int *counter, cudaStream_t st);
void launch_batch_edge(const BatchScene *B, int nb, const int *order, int spt, int ctas_per_sm, int *counter,
                       bool wide, cudaStream_t st);
// Signed distance output (forward: sdf, backward: d_sdf).
void launch_sdf(const DevScene &S, const DevRender &R, const float *eval_positions, int num_eval, float *sdf,
                const float *d_sdf, cudaStream_t st);

}  // namespace dvg

#define DVG_EFLAG_BIN_OVERFLOW 0x100u
