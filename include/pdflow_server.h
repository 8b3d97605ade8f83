/*
 * pdflow_server.h - request loop of the GB300 PD-Flow solver for many live
 * camera streams (no counterpart in the reference, whose live application
 * solves one camera's frames in a single-threaded loop).
 *
 * Streams are admitted against a device-memory budget.  Each admitted stream
 * owns a slot of a "lane": a batch handle with its own CUDA stream and host
 * worker thread, whose slots keep each stream's newest frame pyramid on the
 * device, so a new frame is decoded once and paired with the resident
 * previous one.  A lane that is idle takes, at once, the oldest pending frame
 * of every one of its streams that has one and solves them as one batch
 * (plain, or with the learned warm start); frames that arrive meanwhile wait
 * for the lane's next batch (continuous batching), and lanes run concurrently
 * on the GPU.  Per-pair results do not depend on what else is in the batch.
 * A lane captures its CUDA graphs for every batch size when it is created
 * (on blank frames), so admission, not a live request, pays for them.
 */
#ifndef PDFLOW_SERVER_H
#define PDFLOW_SERVER_H

#include <stddef.h>
#include <stdint.h>

#include "pdflow.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pdflow_server pdflow_server;

typedef struct pdflow_server_config {
    size_t device_budget_bytes;   /* admission limit for all lanes' device memory (solver + network) */
    unsigned slots_per_lane;      /* streams per lane = batch capacity (1..64) */
    int learned;                  /* 1: solve with the learned warm start (net_params required) */
    float iter_scale;             /* learned path: iteration scale */
    float energy_margin;          /* learned path: fallback margin (< 0: never) */
    const float* net_params;      /* network parameters (pdflow_net.h layout), copied at create */
    size_t net_param_count;
} pdflow_server_config;

typedef struct pdflow_request_info {
    unsigned long long request_id;
    unsigned stream_id;
    unsigned long long frame_index;   /* 0-based frame number within its stream */
    int status;                       /* PDFLOW_OK or the error of its batch */
    int has_flow;                     /* 0 for a stream's first frame (nothing to pair with) */
    unsigned batch_pairs;             /* pairs solved in its batch */
    unsigned batch_fallbacks;         /* pairs of its batch re-solved by the plain schedule */
    double submit_ms, start_ms, done_ms;   /* since the server was created (steady clock) */
} pdflow_request_info;

typedef struct pdflow_server_stats {
    unsigned lanes, streams;
    unsigned long long submitted, completed, batches, pairs_solved, fallbacks;
    size_t device_bytes;
} pdflow_server_stats;

int pdflow_server_create(const pdflow_server_config* cfg, pdflow_server** out);
/* Waits for all submitted frames, stops the workers and frees everything. */
int pdflow_server_destroy(pdflow_server* srv);

/* Admits a stream of width x height frames (640x480 -> rows 480, 320x240 ->
 * rows 240): PDFLOW_ERR_OOM when no lane has a free slot and a new lane
 * would exceed the budget. */
int pdflow_server_open_stream(pdflow_server* srv, unsigned width, unsigned height, unsigned* stream_id);
/* Releases a stream's slot; PDFLOW_ERR_STATE while it has frames in flight. */
int pdflow_server_close_stream(pdflow_server* srv, unsigned stream_id);

/* Queues the stream's next frame (row-major uint8 intensity, uint16 depth,
 * copied before returning). */
int pdflow_server_submit(pdflow_server* srv, unsigned stream_id, const uint8_t* intensity, const uint16_t* depth,
                         unsigned long long* request_id);

/* Waits up to timeout_ms (< 0: forever) for the request, then fills *info and,
 * when the request has a flow, dx/dy/dz [rows*cols] (any may be NULL), and
 * forgets the request.  PDFLOW_ERR_TIMEOUT if it is not done in time. */
int pdflow_server_wait(pdflow_server* srv, unsigned long long request_id, int timeout_ms, pdflow_request_info* info,
                       float* dx, float* dy, float* dz);

int pdflow_server_get_stats(pdflow_server* srv, pdflow_server_stats* stats);

/* A camera stream's recorded frames for pdflow_server_replay: frame k is
 * intensity[k] / depth[k] (host, row-major, the stream's size). */
typedef struct pdflow_replay_stream {
    unsigned stream_id;
    unsigned frames;
    const uint8_t* const* intensity;
    const uint16_t* const* depth;
} pdflow_replay_stream;

/* Load generator (no counterpart in the reference): replays the streams'
 * frames with Poisson arrivals, each stream's gaps exponential of mean
 * 1 / rate_hz (seeded), from a generator thread that sleeps until each
 * arrival and submits it, then waits for every request.  info[m] and
 * late_ms[m] (how late submission m was against its schedule) are filled in
 * submission order, *count of them (at most `capacity`: PDFLOW_ERR_ARG when
 * the streams hold more frames).  An error from a submission ends the
 * replay after waiting for the requests already submitted. */
int pdflow_server_replay(pdflow_server* srv, const pdflow_replay_stream* streams, unsigned n_streams, double rate_hz,
                         unsigned long long seed, pdflow_request_info* info, double* late_ms, unsigned capacity,
                         unsigned* count);

#ifdef __cplusplus
}
#endif
#endif /* PDFLOW_SERVER_H */
