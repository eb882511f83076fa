/*
 * TEST INFRASTRUCTURE ONLY — the CPU oracle of diffvg_gb300.
 *
 * A plain-C restatement of the reference's render path (diffvg.cpp,
 * scene.cpp, winding_number.h, within_distance.h, compute_distance.h,
 * sample_boundary.h, solve.h, filter.h, pcg.h, cdf.h) over the packed scene
 * layout of include/diffvg_gb300.h, with parameters in host memory.  Only the
 * test suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * as the checker; the product path never links or calls it.
 */
#ifndef DVG_ORACLE_H
#define DVG_ORACLE_H

#include "../include/diffvg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct DvgOracleArgs {
  int32_t width, height, num_samples_x, num_samples_y;
  uint64_t seed;
  int32_t use_prefiltering;
  int32_t num_threads;            /* <=0: one thread                          */
  const float *params;            /* [num_params]                             */
  const float *background;        /* [h*w*4] or NULL                          */
  const float *eval_positions;    /* [n*2] or NULL                            */
  int32_t num_eval_positions;
  /* forward outputs (accumulated with +=, caller zeroes) */
  float *image;                   /* [h*w*4] or NULL                          */
  float *sdf;                     /* [h*w] / [n] or NULL                      */
  /* backward inputs / outputs */
  const float *d_image;           /* [h*w*4] or NULL                          */
  const float *d_sdf;             /* [h*w] / [n] or NULL                      */
  float *d_params;                /* [num_params] or NULL                     */
  float *d_background;            /* [h*w*4] or NULL                          */
  float *d_translation;           /* [h*w*2] or NULL                          */
  /* diagnostics */
  int64_t *counters;              /* optional [8]: see dvg_oracle.c           */
} DvgOracleArgs;

/* Runs one render call (forward and/or backward, like diffvg.render).
 * Returns DVG_OK or a negative DvgStatus with a message in err. */
int dvg_oracle_render(const DvgSceneDesc *desc, const DvgOracleArgs *args,
                      char *err, int err_len);

#ifdef __cplusplus
}
#endif
#endif
