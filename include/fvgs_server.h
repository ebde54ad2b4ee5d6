/*
 * fvgs_server.h -- serving many SLAM sessions on one GPU (C-ABI).
 *
 * No reference counterpart: the reference tracks a single map, one frame at a
 * time (GSSlam, src/GSSlam.cu).  A server admits sessions (fvgs_session, each
 * with its own Gaussians, frame size and pose state in HBM) against a memory
 * budget and runs their tracking / mapping requests with continuous batching:
 * a session's requests run in order, different sessions' frames overlap on the
 * device (at most max_inflight at a time), each through fvgs_frame_submit on
 * the session's own stream.  While admitted, a session is driven by the
 * server's worker thread only.
 */
#ifndef FVGS_SERVER_H
#define FVGS_SERVER_H

#include "fvgs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fvgs_server fvgs_server;

typedef struct fvgs_server_request {
    fvgs_pose pose;        /* initial pose of the frame */
    fvgs_intrinsics K;
    int level;             /* pyramid level whose frame (fvgs_set_frame) is tracked */
    int iterations;        /* Gauss-Newton iterations */
    float map_eta;         /* >= 0: a mapping step with this learning rate follows */
    uint64_t tag;          /* caller's request id, returned with the result */
    double t_arrival;      /* arrival time (fvgs_server_now clock); <= 0: time of submission */
    /* Optional new observed frame for `level` (as fvgs_set_frame; host
     * memory should be pinned so the copies overlap): copied to the device on
     * the session's stream right before the frame.  rgb == NULL: keep the
     * session's current frame.  The buffers must stay valid until the result
     * is returned. */
    const float* rgb;
    const float* depth;
    const float* grad_x;
    const float* grad_y;
    int width, height;
    /* Optional raw camera frame instead (as fvgs_preprocess_frame: 8-bit
     * colour, float metres or uint16 millimetre depth): the pyramid levels
     * 0..raw_levels-1 are built on the device right before the frame.  Used
     * when raw_color != NULL and rgb == NULL. */
    const uint8_t* raw_color;
    const void* raw_depth;
    int raw_depth_u16_mm;
    int raw_levels;
    int raw_double_scale;
    /* Coarse-to-fine frame instead of one level: when pyr_levels > 0, K is
     * the level-0 intrinsics and the frame runs pyr_iterations[l] steps at
     * every level l < pyr_levels from the coarsest down (as
     * fvgs_frame_submit_pyramid); level and iterations are then unused. */
    int pyr_levels;
    int pyr_iterations[FVGS_MAX_LEVELS];
    /* Optional observed frames of levels 0..pyr_levels-1 (with pyr_levels >
     * 0; used instead of rgb / raw_color), packed one level after the other,
     * each as rgb[3P], depth[P], grad_x[3P], grad_y[3P] with P = W_l H_l,
     * W_0 = width, H_0 = height, W_{l+1} = (W_l + 1) / 2, H_{l+1} =
     * (H_l + 1) / 2: one host buffer (pinned, so the copies overlap) copied to
     * the device on the session's stream right before the frame. */
    const float* pyr_frames;
} fvgs_server_request;

typedef struct fvgs_server_result {
    uint64_t tag;
    int slot;
    int status;            /* fvgs_status of the frame */
    fvgs_pose pose;        /* tracked pose */
    double last_step[6];
    double t_arrival, t_launch, t_done;  /* fvgs_server_now clock, seconds */
} fvgs_server_result;

int fvgs_server_create(uint64_t memory_budget_bytes, int max_inflight, fvgs_server** out);
/* Waits for queued and running frames, then stops the worker. */
int fvgs_server_destroy(fvgs_server* sv);
/* Admit a session if the admitted footprints (fvgs_session_footprint) fit the
 * budget; FVGS_E_ADMISSION otherwise. */
int fvgs_server_admit(fvgs_server* sv, fvgs_session* s, int* slot);
/* Waits for the session's frames, then frees its share of the budget. */
int fvgs_server_release(fvgs_server* sv, int slot);
int fvgs_server_submit(fvgs_server* sv, int slot, const fvgs_server_request* req);
/* Up to max_results completed frames, in completion order; waits until at
 * least wait_for are available (or nothing more can complete). */
int fvgs_server_results(fvgs_server* sv, fvgs_server_result* out, int max_results, int wait_for, int* n);
int fvgs_server_now(double* seconds);
int fvgs_server_stats(fvgs_server* sv, uint64_t* admitted_bytes, int* inflight, uint64_t* launched,
                      uint64_t* completed);

#ifdef __cplusplus
}
#endif

#endif /* FVGS_SERVER_H */
