/* fastjet_gb300: GB300-native sequential-recombination jet clustering.
 *
 * C ABI of libfastjet_gb300.so.  All entry points return an fjg_status and
 * never abort.  Buffers are owned by the caller; device pointers must be
 * device-accessible on the context's device.  Calls that take a stream are
 * stream-ordered (asynchronous with respect to the host) unless stated.
 *
 * Reference interface replaced (fwyzard/fastjet_gpu):
 *   cluster.h:4   enum class Algorithm { Kt = 1, CambridgeAachen = 0, AntiKt = -1 }
 *                 -> FJG_KT / FJG_CAM / FJG_ANTIKT (same values, the exponent p)
 *   PseudoJet.h:4 struct PseudoJet { int index; bool isJet; double px, py, pz, E; }
 *                 -> fjg_pseudojet (identical layout, 40 bytes)
 *   cluster.h:6   void cluster(PseudoJet *particles, int size, Algorithm algo, double r)
 *                 -> fjg_cluster_pseudojets (same in-place device-buffer contract),
 *                    and the unchanged C++ symbol in fastjet_gb300_compat.h
 *   main.cc:269-335 per-event loop of the driver (H2D copy, cluster, D2H copy,
 *                 isJet/ptmin filter, pT sort)
 *                 -> fjg_cluster_batch / fjg_cluster_batch_host for many events
 *                    per call, fjg_serve_* for events arriving over time.
 */
#ifndef FASTJET_GB300_H
#define FASTJET_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FJG_OK = 0,
  FJG_EINVAL = 1,     /* invalid argument (null pointer, bad algorithm, negative size, R <= 0) */
  FJG_ENOMEM = 2,     /* device or host allocation failed */
  FJG_ECUDA = 3,      /* a CUDA runtime call failed; fjg_last_error() has the message */
  FJG_ETOOBIG = 4,    /* an event exceeds the supported particle count */
  FJG_ETIMEDOUT = 5,  /* a bounded device wait ran out (serving queue) */
  FJG_EAGAIN = 6,     /* serving: no free slot or result not ready yet */
  FJG_EKERNEL = 7     /* a kernel reported an internal inconsistency */
} fjg_status;

/* Algorithm codes: the reference enum values (cluster.h:4). */
#define FJG_KT 1
#define FJG_CAM 0
#define FJG_ANTIKT (-1)

/* Largest event the library clusters (particles per event); larger events
 * are refused with FJG_ETOOBIG.  Events above 4096 particles also need the
 * tiled kernel's workspace (96 bytes per particle of the batch). */
#define FJG_MAX_EVENT_PARTICLES 16777216

/* I/O record of the reference (PseudoJet.h:4-11): 40 bytes, px at offset 8. */
typedef struct {
  int index;
#ifdef __cplusplus
  bool isJet;
#else
  _Bool isJet;
#endif
  double px, py, pz, E;
} fjg_pseudojet;

/* One clustering step: a merge of pseudojets a < b, or (b == -1) the promotion
 * of a to a final jet; d is the winning distance.  A pseudojet's label is the
 * lowest input index among its constituents. */
typedef struct {
  int32_t a;
  int32_t b;
  double d;
} fjg_step;

/* Outputs of a batch, CSR-indexed by the batch's offsets (event e owns
 * [offsets[e], offsets[e+1])).  Jets of event e are jets[offsets[e] + k],
 * k < n_jets[e], in promotion order; rows of jets and jet_label past
 * n_jets[e] are left unspecified (not cleared).  history and owner may be NULL. */
typedef struct {
  double* jets;       /* [total][4] px, py, pz, E */
  int32_t* jet_label; /* [total] label of each jet */
  int32_t* n_jets;    /* [n_events] */
  fjg_step* history;  /* [total] optional: one record per step */
  int32_t* owner;     /* [total] optional: for each input particle, index k of its jet */
} fjg_outputs;

typedef struct fjg_ctx fjg_ctx;

/* Create a context on `device` (a CUDA ordinal).  The context owns a stream,
 * cached scratch memory and captured CUDA graphs.  Thread-safe per context
 * only under external serialisation. */
fjg_status fjg_ctx_create(int device, fjg_ctx** out);
void fjg_ctx_destroy(fjg_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t). */
void* fjg_ctx_stream(fjg_ctx* ctx);
const char* fjg_status_string(fjg_status s);
/* Wait for the context's work and report (then clear) errors raised by its
 * kernels since the last check, e.g. FJG_ETOOBIG from an asynchronous batch. */
fjg_status fjg_ctx_check(fjg_ctx* ctx);
/* Last error message of the context (or of the calling thread when ctx is NULL). */
const char* fjg_last_error(const fjg_ctx* ctx);
/* Per-step phase counters of the clustering kernels, summed over the events
 * clustered through this context's batch and one-event calls.  Shared-memory
 * kernel: out[0..3] clock cycles in the argmin, merge, new-jet and
 * neighbour-resolution phases as the CTA's thread 0 sees them, out[4..6] in
 * the merge warps' kinematics chains, out[7] in the first rescan thread's
 * merge-phase work, out[8] steps, out[9] events, out[10], out[11], out[22],
 * out[23] how many FP64 fallbacks the argmin, the closer-neighbour tests, the
 * key updates and the neighbour searches took.  Tiled kernel (events above
 * 4096 particles): out[12..17] cycles in the list rebuilds, the argmin, the
 * merge and target detection, the list update with the targets and the new
 * jet's window pass, the pass for targets beyond the listed ones, the tile
 * summaries; out[18] in the rapidity chain, out[19] in the first detection
 * thread's merge-phase work, out[20] steps, out[21] events, out[24] targets
 * found (slots whose neighbour was merged) and out[25] steps with any;
 * out[26..28] thread 0's list update, warp 1's targets and thread 0's share
 * of the window pass; out[29..31] warp 0's resolution of the new jet's
 * neighbour and its merge into its tile's summary, and warp 1's summary work
 * (n <= 32 entries).  Only a library built with
 * -DFJG_PHASE_CLOCKS (python -m fastjet_gpu_gb300.build --phase-clocks) has
 * them; the product build returns FJG_EINVAL.  Waits for the context stream;
 * `reset` zeroes them.  No counterpart in the reference. */
fjg_status fjg_phase_clocks(fjg_ctx* ctx, unsigned long long* out, int n, int reset);

/* Batched clustering of device-resident events (the persistent-kernel path).
 *   p4      device [total][4] FP64 px, py, pz, E
 *   offsets device [n_events + 1] int64, offsets[0] == 0
 *   algo    device [n_events] int32 or NULL (then algo_all for every event)
 *   radius  device [n_events] FP64 or NULL (then r_all for every event)
 *   total   offsets[n_events] (host value; sizes the scratch)
 *   stream  cudaStream_t or NULL for the context stream
 * Events are clustered independently; results do not depend on batch
 * composition. */
fjg_status fjg_cluster_batch(fjg_ctx* ctx, const double* p4, const int64_t* offsets, int n_events, int64_t total,
                             const int32_t* algo, int algo_all, const double* radius, double r_all,
                             const fjg_outputs* out, void* stream);

/* Same, with every buffer in host memory (pinned or pageable).  Copies the
 * inputs to the device, clusters, copies the outputs back, and synchronises. */
fjg_status fjg_cluster_batch_host(fjg_ctx* ctx, const double* p4, const int64_t* offsets, int n_events,
                                  const int32_t* algo, int algo_all, const double* radius, double r_all,
                                  const fjg_outputs* out);

/* The plain path: one event per launch on the context stream, one CTA,
 * synchronous.  Device buffers as in fjg_cluster_batch for a single event. */
fjg_status fjg_cluster_event(fjg_ctx* ctx, const double* p4, int n, int algo, double r, double* jets,
                             int32_t* jet_label, int32_t* n_jets, fjg_step* history, int32_t* owner);

/* Rapidity, azimuth in [0, 2pi) and clustering weight (kt: pt^2, C/A: 1,
 * anti-kt: 1/pt^2) of n device four-momenta, as the clustering kernels compute
 * them; replaces the reference's per-particle _set_jet (tri_matrix.cu:61-100,
 * grid.cu:112-171).  Asynchronous on `stream` (NULL: the context stream). */
fjg_status fjg_kinematics(fjg_ctx* ctx, const double* p4, int n, int algo, double* rap, double* phi, double* w,
                          void* stream);

/* Drop-in for the reference's cluster() (cluster.h:6): `particles` is a device
 * buffer of `size` records, rewritten in place.  On return every record has
 * index = its input position; records whose slot holds a final jet have
 * isJet = true and the jet's momentum (the jet sits at the slot of its
 * lowest-index constituent); all other records have isJet = false.
 * Synchronous on the given stream (NULL: the context stream). */
fjg_status fjg_cluster_pseudojets(fjg_ctx* ctx, fjg_pseudojet* particles, int size, int algo, double r,
                                  void* stream);

/* ------------------------------------------------------------ epilogue
 * Replaces the reference driver's host post-processing (main.cc:309-327):
 * per event, keep the inclusive jets with px*px + py*py >= ptmin^2 and, when
 * `sort` is nonzero, order them by decreasing pt^2 (equal pt^2 by increasing
 * jet label; the reference's std::sort leaves that order unspecified).
 * Inputs are a batch's outputs (device memory, CSR by `offsets`, `total` =
 * offsets[n_events]); outputs go to the same positions of out_jets /
 * out_label, with the kept count in out_n_jets.  Stream-ordered. */
fjg_status fjg_select_jets(fjg_ctx* ctx, const double* jets, const int32_t* jet_label, const int32_t* n_jets,
                           const int64_t* offsets, int n_events, int64_t total, double ptmin, int sort,
                           double* out_jets, int32_t* out_label, int32_t* out_n_jets, void* stream);

/* The driver's --combine k (main.cc:76-85, 269) on a device CSR batch: every
 * k consecutive events become one (k = 0: all of them), which only changes
 * the offsets -- out_offsets[i] = offsets[min(i k, n_events)] for
 * i = 0 .. *n_out, with *n_out = ceil(n_events / k).  Stream-ordered;
 * *n_out is known on return. */
fjg_status fjg_combine_events(fjg_ctx* ctx, const int64_t* offsets, int n_events, int k, int64_t* out_offsets,
                              int* n_out, void* stream);

/* ------------------------------------------------------------ CUDA graphs
 * No counterpart in the reference (one synchronous call per event).
 *
 * fjg_graph_capture_batch records one fjg_cluster_batch call on these device
 * buffers (bucketing kernels, the per-bucket persistent kernels and the tiled
 * kernel, with their fork/join across the context's side streams) as a CUDA
 * graph.  n_events and total are fixed by the capture; the buffers' contents
 * -- momenta, offsets (event sizes), per-event algorithms and radii -- may
 * change between launches as long as offsets[n_events] <= total.  The graph
 * owns its scratch, so graphs of one context may run concurrently on
 * different streams; a graph's own launches must not overlap each other.  The
 * context's tuning at capture time is baked in. */
typedef struct fjg_graph fjg_graph;
fjg_status fjg_graph_capture_batch(fjg_ctx* ctx, const double* p4, const int64_t* offsets, int n_events,
                                   int64_t total, const int32_t* algo, int algo_all, const double* radius,
                                   double r_all, const fjg_outputs* out, fjg_graph** graph);
/* Launch on `stream` (NULL: the context's stream); asynchronous. */
fjg_status fjg_graph_launch(fjg_graph* graph, void* stream);
/* Wait for the last launch and report the kernels' status (FJG_ETOOBIG,
 * FJG_EKERNEL, FJG_EINVAL for bad offsets); clears it. */
fjg_status fjg_graph_check(fjg_graph* graph);
void fjg_graph_destroy(fjg_graph* graph);

/* ------------------------------------------------------------ autotuning
 * No counterpart in the reference.  The batch launcher runs events of up to
 * 256, 512, 1024, 2048 and 4096 particles (buckets 0-4) with one of several
 * compiled kernel shapes each (CTA threads x slots per thread = the bucket's
 * capacity) and a persistent grid of ctas_per_sm CTAs per SM (0: as many as
 * fit); events above 4096 particles run on the tiled kernel with a grid of
 * large_ctas_per_sm CTAs per SM (one is resident per SM) and rapidity-azimuth
 * tiles of side at least tile_factor * R (tile_factor >= 1), larger where an
 * event is sparse (about 32 particles per tile).  Every choice gives identical
 * results; only the speed differs. */
#define FJG_NUM_BUCKETS 5
typedef struct {
  int32_t threads[FJG_NUM_BUCKETS];          /* CTA size: 64 .. 512 */
  int32_t slots_per_thread[FJG_NUM_BUCKETS]; /* threads * slots_per_thread = 256 << bucket */
  int32_t ctas_per_sm[FJG_NUM_BUCKETS];      /* 0: the occupancy limit */
  double events_per_s[FJG_NUM_BUCKETS];      /* the autotuner's measurement (0 when set by hand) */
  int32_t large_ctas_per_sm;   /* 1 .. 8 */
  double tile_factor;          /* 1 .. 8 */
} fjg_tuning;

fjg_status fjg_get_tuning(fjg_ctx* ctx, fjg_tuning* tuning);
/* FJG_EINVAL if a (threads, slots_per_thread) pair is not one of the compiled
 * shapes of that bucket's capacity or a field is out of range. */
fjg_status fjg_set_tuning(fjg_ctx* ctx, const fjg_tuning* tuning);
/* Time every compiled shape and a few CTA-per-SM counts on synthetic events
 * of each bucket's size range for `algo` and `r`, keep the fastest, and
 * return the choice in *result (may be NULL).  The tiled kernel's tile side
 * follows each event's particle density (at least R), so tile_factor is set
 * to 1; FJG_TUNE_SKIP_LARGE is accepted and has no effect.  Takes about a
 * second per bucket; synchronous. */
#define FJG_TUNE_SKIP_LARGE 1
fjg_status fjg_autotune(fjg_ctx* ctx, int algo, double r, int flags, fjg_tuning* result);

/* ------------------------------------------------------------ event text
 * Reads the reference driver's input format (main.cc:34-70) into CSR arrays:
 * one particle per line, "px py pz E" (whitespace separated; anything after
 * the fourth number is ignored); an event is a maximal run of such lines; an
 * empty line or one starting with '#' ends an event; any other line is
 * rejected, as the reference's reader throws on it; a final line without a
 * newline is not read (the reference's getline loop stops there).  Numbers are correctly
 * rounded decimals with an optional sign (no inf/nan), the values
 * istream >> double gives.  `particles` receives [n_particles][4] doubles,
 * `offsets` n_events + 1 entries (offsets[0] = 0).  Host only: no context or
 * device is involved; `threads` <= 0 uses every hardware thread (texts below
 * 1 MiB are read by one).  FJG_EINVAL with *error_line (1-based) on a rejected
 * line; FJG_ETOOBIG when max_particles or max_offsets is too small, with
 * *n_particles and *n_events set to what is needed.  Replaces the driver's
 * read_n_events (main.cc:76-85) for callers of the library. */
fjg_status fjg_parse_events(const char* text, size_t len, int threads, double* particles, int64_t max_particles,
                            int64_t* offsets, int64_t max_offsets, int64_t* n_particles, int64_t* n_events,
                            int64_t* error_line);

/* ------------------------------------------------------------ serving
 * No counterpart in the reference.  A request server on one context: events
 * are submitted one at a time as they arrive and complete independently.
 *
 * - State: a particle arena of `arena_particles` entries.  An admitted event
 *   holds a contiguous range of it: its momenta are copied into device memory
 *   as it is admitted (through a pinned staging range) and stay there with its
 *   clustering state (the FP64 workspace, and the tiled kernel's workspace
 *   above 4096 particles) while it is clustered; its results go to pinned host
 *   memory that the kernels write directly.  Admission is first come, first served, by
 *   arena space (the HBM footprint) and by the resident CTA slots of the
 *   event's size bucket (the shared-memory footprint, oversubscribed by at
 *   most `oversubscribe`).
 * - Continuous batching: admitted events of one size bucket are launched
 *   together as a micro-batch on the first idle stream of a pool of
 *   `streams`, smallest buckets first, while earlier micro-batches are still
 *   running; events above 4096 particles use at most half of the streams and
 *   have at most one in flight per two SMs, so that they cannot keep the
 *   small requests off the GPU; every event
 *   raises its own completion flag in mapped host memory as soon as it is
 *   done, so results do not wait for the rest of their micro-batch.
 * - Progress happens inside fjg_server_submit and fjg_server_poll (no
 *   background thread); a server is driven by one host thread at a time.
 * Results are identical to fjg_cluster_batch on the same event. */
typedef struct fjg_server fjg_server;
typedef struct {
  int64_t arena_particles; /* default 4194304 */
  int32_t max_inflight;    /* events admitted and not yet released; default 8192 */
  int32_t streams;         /* micro-batch streams; default 16 */
  int32_t max_batch;       /* events per micro-batch; default 512 */
  int32_t oversubscribe;   /* launched events per resident CTA slot of a bucket; default 2 */
  int32_t flags;           /* FJG_SERVE_HISTORY, FJG_SERVE_DEVICE_CHECK (below) */
} fjg_server_config;
/* Also return the merge history and constituents of every request. */
#define FJG_SERVE_HISTORY 1
/* Check momenta for NaN/inf on the GPU, as a micro-batch is launched, instead
 * of on the host at submission (which costs a pass over the request on the
 * submitting thread).  A request that fails the check completes with status
 * FJG_EINVAL and no jets; the other requests of its micro-batch are clustered
 * as usual. */
#define FJG_SERVE_DEVICE_CHECK 2

/* One completed request.  The pointers are into the server's arena and stay
 * valid until fjg_server_release(ticket). */
typedef struct {
  uint64_t ticket;
  int32_t status;          /* FJG_OK, or this request's own error (FJG_EINVAL: refused input;
                              FJG_EKERNEL: a kernel inconsistency); a failed request does
                              not affect the others */
  int32_t n_particles;
  int32_t n_jets;
  const double* jets;      /* [n_jets][4], in promotion order */
  const int32_t* jet_label;
  const fjg_step* history; /* [n_particles] or NULL */
  const int32_t* owner;    /* [n_particles] or NULL */
  double latency_us;       /* from submission to the completion being observed */
} fjg_served;

/* config may be NULL (defaults); zero fields take their defaults. */
fjg_status fjg_server_create(fjg_ctx* ctx, const fjg_server_config* config, fjg_server** server);
void fjg_server_destroy(fjg_server* server);
/* Queue one event (host memory, [n][4] px py pz E; copied); FJG_EINVAL for
 * bad arguments, FJG_ETOOBIG when it can never fit the arena. */
fjg_status fjg_server_submit(fjg_server* server, const double* p4, int n, int algo, double r, uint64_t* ticket);
/* Make progress and return up to `max` completed requests; waits up to
 * timeout_us microseconds for the first one (0: do not wait). */
fjg_status fjg_server_poll(fjg_server* server, fjg_served* out, int max, int* n_out, int64_t timeout_us);
/* Free the arena range of a returned request. */
fjg_status fjg_server_release(fjg_server* server, uint64_t ticket);
/* Submitted and not yet returned by fjg_server_poll. */
int fjg_server_pending(const fjg_server* server);
/* Clustering kernels launched by the server so far (one per micro-batch). */
int64_t fjg_server_launches(const fjg_server* server);
/* Open-loop replay of a request trace (benchmarking): event i (CSR p4 and
 * offsets in host memory, algo[i], radius[i]) is submitted at arrival_us[i]
 * microseconds after the start, results are released as they complete, and
 * latency_us[i] receives the time from the scheduled arrival to the observed
 * completion.  *wall_us receives the time to the last completion. */
fjg_status fjg_server_replay(fjg_server* server, const double* p4, const int64_t* offsets, int n_events,
                             const int32_t* algo, const double* radius, const double* arrival_us,
                             double* latency_us, double* wall_us);

/* Batched clustering that allocates no memory (no counterpart in the
 * reference, which allocates on every call).  For callers that cannot call
 * cudaMalloc at this point -- real-time or trigger code that forbids
 * allocation after initialisation (an allocation can synchronise the device
 * and take unbounded time), or an application whose device memory belongs to
 * another allocator or a quota -- and that therefore cannot create a context
 * either.  Arguments as in fjg_cluster_batch, all device buffers supplied by
 * the caller; runs on `stream` (NULL: the legacy default stream) on the
 * current device and returns after synchronising it.
 * Limits: at most FJG_NOALLOC_MAX_EVENTS events and FJG_NOALLOC_MAX_PARTICLES
 * particles (`total` = offsets[n_events]) per call (larger batches return
 * FJG_EINVAL).  The
 * kernels' bookkeeping and per-particle working state live in a static device
 * array of FJG_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds
 * until exit.  The first call on each device also looks up that array's
 * address.  Every call synchronises `stream` before it returns (it reads the
 * kernels' status word back), so the entry point cannot be used inside stream
 * capture.  Calls share the array: calls whose work overlaps on the GPU race
 * and must be serialised by the caller.  Event ranges outside [0, total) are
 * refused (FJG_EINVAL) and their momenta are not read, as are non-finite
 * momenta. */
#define FJG_NOALLOC_MAX_EVENTS 65536
#define FJG_NOALLOC_MAX_PARTICLES 131072
#define FJG_NOALLOC_SCRATCH_BYTES ((7 * 8 + 96) * FJG_NOALLOC_MAX_PARTICLES + 6 * 4 * FJG_NOALLOC_MAX_EVENTS + 32768)
fjg_status fjg_cluster_batch_noalloc(const double* p4, const int64_t* offsets, int n_events, int64_t total,
                                     const int32_t* algo, int algo_all, const double* radius, double r_all,
                                     const fjg_outputs* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FASTJET_GB300_H */
