/*
 * gbopticks.h : C ABI of the GB300 optical-photon engine (libgbopticks.so).
 *
 * Plain pointers and sizes only.  Every entry point returns GBO_OK (0) or an error code; the message of the
 * calling thread's last error is available from gbo_last_error().  Array layouts are those of gbo_types.h,
 * i.e. the reference's own genstep / photon / CSGFoundry layouts.
 *
 * Reference interface each entry point stands in for:
 *
 *   gbo_config_default   SEventConfig defaults + OPTICKS_* environment (sysrap/SEventConfig.cc:37-115,
 *                        keys sysrap/SEventConfig.hh:218-283)
 *   gbo_engine_create    G4CXOpticks::SetGeometry(const G4VPhysicalVolume*) (g4cx/G4CXOpticks.hh:49,
 *                        g4cx/G4CXOpticks.cc:79-84, 315-346): geometry + optical tables uploaded once; the caller
 *                        has already translated the Geant4 tree into CSGFoundry arrays (CSG/CSGFoundry.cc:2782-2788)
 *   gbo_simulate         G4CXOpticks::simulate(int eventID, bool reset=false) (g4cx/G4CXOpticks.hh:95,
 *                        .cc:466-486) with gensteps that SEvt::AddGenstep collected (sysrap/SEvt.hh:487) and the
 *                        input photons of SEvt::SetInputPhoton; synchronous, hits gathered when it returns
 *   gbo_simulate_to_host G4CXOpticks::simulate followed by the gather of the event's hits into host memory
 *                        (QSim::simulate gathers each genstep slice's hits in turn, qudarap/QSim.cc:481-529), in one
 *                        call
 *   gbo_num_hit          SEvt::GetNumHit(0) (sysrap/SEvt.cc:2050)
 *   gbo_copy_hits        SEvt::getHit(sphoton&, unsigned idx) (sysrap/SEvt.cc:4991), in bulk
 *   gbo_reset            G4CXOpticks::reset(int eventID) (g4cx/G4CXOpticks.hh:96, .cc:499-518)
 *   gbo_copy_photons     the full photon array of a debug event mode (QEvt::gatherPhoton)
 *   gbo_copy_seq         the seqhis/seqbnd arrays of a debug event mode (sysrap/sseq.h)
 *   gbo_simulate_device  QSim::simulate on gensteps already resident in device memory (qudarap/QSim.cc:428-631)
 *   gbo_engine_destroy   G4CXOpticks::Finalize
 */
#ifndef GBOPTICKS_H
#define GBOPTICKS_H

#include <stdint.h>
#include "gbo_types.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GBO_OK = 0,
    GBO_ERR_ARG = 1,        /* bad argument (null pointer, size out of range, malformed geometry) */
    GBO_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    GBO_ERR_STATE = 3,      /* call out of order (e.g. hits requested before any simulate) */
    GBO_ERR_CAPACITY = 4,   /* request above a configured or fixed limit */
    GBO_ERR_DEVICE = 5,     /* a kernel reported an error through its status word, or a served event failed */
    GBO_ERR_TIMEOUT = 6     /* gbo_server_wait ran out of time; the event is still in flight */
};

typedef struct gbo_engine gbo_engine;

typedef struct gbo_geometry_desc {
    const gbo_csgnode*  node;    int32_t num_node;
    const gbo_csgprim*  prim;    int32_t num_prim;
    const gbo_csgsolid* solid;   int32_t num_solid;
    const gbo_qat4*     inst;    int32_t num_inst;     /* forward transforms, identity ints in .w column */
    const gbo_qat4*     itra;    int32_t num_itra;     /* inverse node transforms (1-based gtransformIdx) */
    const float*        plan;    int32_t num_plan;     /* float4 planes */
    const float*        bnd;     int32_t num_bnd;      /* (num_bnd, 4, 2, bnd_nx, 4) boundary payload */
    int32_t             bnd_nx;                        /* wavelength samples (761) */
    float               bnd_domain_low;                /* nm (60) */
    float               bnd_domain_step;               /* nm (1) */
    const uint32_t*     optical;                       /* (num_bnd*4, 4) */
    const float*        icdf;                          /* (icdf_ny, icdf_nx) scintillation inverse CDF */
    int32_t             icdf_ny, icdf_nx, hd_factor;
} gbo_geometry_desc;

typedef struct gbo_config {
    int32_t  max_bounce;            /* OPTICKS_MAX_BOUNCE        31    */
    float    max_time;              /* OPTICKS_MAX_TIME          1e27 ns */
    float    propagate_epsilon;     /* OPTICKS_PROPAGATE_EPSILON 0.05 mm */
    float    propagate_epsilon0;    /* OPTICKS_PROPAGATE_EPSILON0 0.05 mm */
    uint32_t epsilon0_mask;         /* OPTICKS_PROPAGATE_EPSILON0_MASK TO,CK,SI,SC,RE */
    uint32_t hit_mask;              /* OPTICKS_HIT_MASK          SD    */
    uint64_t rng_seed;              /* QRng__SEED_OFFSET seed    0     */
    uint64_t rng_offset;            /* QRng__SEED_OFFSET offset  0     */
    uint64_t event_skipahead;       /* OPTICKS_EVENT_SKIPAHEAD   100000 */
    float    tmax;                  /* trace limit               1e6 mm */
    int32_t  debug_tag;             /* 1: draw order of the reference's OptiX build (alignment burns), 0: PRODUCTION */
    int32_t  record_photon;         /* keep the full photon array of each event */
    int32_t  record_seq;            /* keep seqhis/seqbnd of each event */
    int64_t  max_photon;            /* capacity limit per event (0: no limit beyond device memory) */
    int32_t  kernel_mode;           /* 0: persistent photon-pool kernel generating its photons, 1: one thread per
                                       photon, 2 (default): photon pool over photons generated up front by a
                                       separate kernel (84 more device bytes per photon), 3: wavefront, every step
                                       of every live photon as three passes (query to the instance-tree walk, the
                                       queued walks, physics) over photons generated up front (136 more device bytes
                                       per photon, 168 in the precision mode).
                                       gbo_simulate_noalloc runs its own one-thread kernel */
    int32_t  refill_min;            /* pool kernel: idle lanes a warp waits for before refilling (1..32, 4) */
    int32_t  blocks_per_sm;         /* pool kernel: resident blocks per SM (0: occupancy maximum) */
    int32_t  refill_period;         /* pool kernel: steps between refill checks (compaction period, >= 1) */
    int64_t  max_slot;              /* OPTICKS_MAX_SLOT: photons per launch, larger events are sliced (0: no slicing) */
    int32_t  precision;             /* 0: binary32 as the reference (default); 1: binary64 Newton polish of every
                                       accepted sphere / zsphere / cylinder root and binary64 position/time
                                       accumulators */
    int32_t  walk_min;              /* pool kernels of geometries with CSG trees: a lane whose step needs a walk of
                                       the instance tree parks until this many lanes of its warp need one (or no other
                                       lane can step), so the walks run together; 1: no parking (1) */
    int32_t  rng_call;              /* kernels of geometries without CSG trees, binary32: 1 (default) computes each
                                       block of four draws by an out-of-line call (smaller code; the CSG-tree kernels
                                       always do), 0 inlines the Philox rounds at every draw site.  Same numbers either
                                       way */
    int32_t  reserved;
} gbo_config;

/* Result of gbo_autotune: the kernel form chosen (kernel mode, refill threshold, refill period = compaction period,
 * resident blocks per SM = block shape with 0 the occupancy maximum, lanes gathered per TLAS walk = walk queue,
 * Philox by call) and the simulate time of every candidate. */
typedef struct gbo_tune_result {
    int32_t kernel_mode, refill_min, refill_period, num_candidates;
    int32_t cand_mode[32], cand_refill[32], cand_period[32];
    float   cand_ms[32];
    int32_t blocks_per_sm;
    int32_t cand_blocks[32];
    int32_t walk_min;
    int32_t cand_walk[32];
    int32_t rng_call;
    int32_t cand_rng_call[32];
} gbo_tune_result;

typedef struct gbo_stats {
    int64_t num_photon;
    int64_t num_hit;
    float   ms_upload;              /* host->device copies of gensteps / input photons */
    float   ms_simulate;            /* simulate kernel */
    float   ms_compact;             /* hit scan + gather */
    int32_t simulate_launches;
    int32_t kernel_launches;        /* all engine kernels of the last event */
    float   ms_generate;            /* kernel mode 2: the generation kernel (part of ms_simulate) */
    int32_t reserved;
} gbo_stats;

int         gbo_config_default(gbo_config* cfg);
int         gbo_engine_create(const gbo_geometry_desc* geom, const gbo_config* cfg, int device, gbo_engine** out);
void        gbo_engine_destroy(gbo_engine* e);
int         gbo_simulate(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                         const gbo_sphoton* input_photon, int64_t num_input_photon);
/* gbo_simulate_to_host : gbo_simulate, then the event's hits (photon order, as gbo_copy_hits gives them) written into
 * `hits`, room for hit_capacity hits (page-locked memory for full copy speed).  With max_slot set the event runs as
 * max_slot slices and each slice's hits are copied out as soon as it ends, on a stream of their own.  Results equal
 * gbo_simulate's for the same event id.  *num_hit receives the hit count; above hit_capacity the call stores the
 * first hit_capacity hits and returns GBO_ERR_CAPACITY.  The event's hits also stay on the device as after
 * gbo_simulate. */
int         gbo_simulate_to_host(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                                 const gbo_sphoton* input_photon, int64_t num_input_photon, gbo_sphoton* hits,
                                 int64_t hit_capacity, int64_t* num_hit);
int         gbo_simulate_device(gbo_engine* e, int32_t event_id, const void* d_gs, int64_t num_gs,
                                const void* d_input_photon, int64_t num_input_photon, void* cuda_stream);
/* gbo_simulate_slice : one launch of a slice of an event, the photons of `gs` being event photons
 * photon_offset + i (the reference's photon_slot_offset, CSGOptiX/CSGOptiX.cc prepareParam, used by QSim::simulate's
 * genstep slices qudarap/QSim.cc:481-529); RNG streams and photon indices are those of the whole event, so slices
 * simulated separately (e.g. on different GPUs) give exactly the photons of the whole event. */
int         gbo_simulate_slice(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                               const gbo_sphoton* input_photon, int64_t num_input_photon, uint64_t photon_offset);
int64_t     gbo_num_hit(const gbo_engine* e);
int64_t     gbo_num_photon(const gbo_engine* e);
int         gbo_copy_hits(gbo_engine* e, gbo_sphoton* dst, int64_t offset, int64_t count);
int         gbo_copy_photons(gbo_engine* e, gbo_sphoton* dst, int64_t offset, int64_t count);
int         gbo_copy_seq(gbo_engine* e, gbo_seq* dst, int64_t offset, int64_t count);
const void* gbo_device_hits(const gbo_engine* e);
/* Hit merging, the reference's per-launch SPM::merge_partial_select (sysrap/SPM.cu, called from QEvt::PerLaunchMerge
 * qudarap/QEvt.cc:1170-1210) with sphoton::key_functor / reduce_op (sysrap/sphoton.h:277-304): the current event's
 * hits grouped by (sensor identity, floor(time / time_window)), each group becoming its earliest hit with the
 * group's flagmasks ORed and hitcounts summed, in ascending key order.  time_window 0 keeps the hits unmerged
 * (NOMERGE_TIME_WINDOW); the reference's OPTICKS_MERGE_WINDOW is typically 1 ns.
 * gbo_merge_hits_device does the same for any device array of n hits into d_out (room for n), on `stream`. */
int         gbo_merge_hits(gbo_engine* e, float time_window, int64_t* num_merged);
int         gbo_copy_merged_hits(gbo_engine* e, gbo_sphoton* dst, int64_t offset, int64_t count);
int         gbo_merge_hits_device(const gbo_sphoton* d_in, int64_t n, float time_window, gbo_sphoton* d_out,
                                  int64_t* num_out, void* stream);
int         gbo_reset(gbo_engine* e, int32_t event_id);
int         gbo_get_stats(const gbo_engine* e, gbo_stats* out);
const char* gbo_last_error(void);

/* gbo_autotune : no counterpart in the reference (its launch shape is fixed by OptiX).  Runs the given sample
 * event with every candidate kernel form (one thread per photon; photon pool with refill thresholds 1..32 and
 * refill periods 1, 4; pool over pregenerated photons with refill thresholds 1..16 and with 16, 24 or 32 lanes
 * gathered per TLAS walk; both pools with fewer resident blocks per SM than fit), `trials` timed runs each after
 * one warm-up, and keeps the fastest in the engine's config.  Every candidate gives the same photons (the kernel
 * form decides only which lane runs a photon, and when). */
int         gbo_autotune(gbo_engine* e, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                         const gbo_sphoton* input_photon, int64_t num_input_photon, int32_t trials,
                         gbo_tune_result* out);

/* Known-answer entry points; the reference drives equivalent test kernels from QSimTest (qudarap/QSim.cu,
 * qudarap/tests/QSimTest.cc:700-770):
 *   gbo_rng_sequence      QSim::rng_sequence : num_seq consecutive subsequences from subsequence0, per_seq
 *                         uniforms each, starting at stream position (offset + skipahead) `position`
 *   gbo_texture_lookup    QBnd / QScint texture lookups at normalized (x,y) pairs; which 0: boundary texture
 *                         (float4 out), 1: scintillation ICDF (value in .x of each float4 out)
 *   gbo_scint_wavelength  qscint::wavelength (hd_factor layers) for each uniform u */
int         gbo_rng_sequence(int device, uint64_t seed, uint64_t subsequence0, uint64_t position, int32_t num_seq,
                             int32_t per_seq, float* out);
int         gbo_texture_lookup(gbo_engine* e, int32_t which, const float* xy, int32_t n, float* out);
int         gbo_scint_wavelength(gbo_engine* e, const float* u, int32_t n, float* out);
/*   gbo_trace_rays        CSGScan (CSG/CSGScan.cu) : closest-hit distance (-1 on a miss) and boundary for n rays
 *                         (pos, dir: n x float3), with the engine's precision setting */
int         gbo_trace_rays(gbo_engine* e, const float* pos, const float* dir, int32_t n, float tmin, float tmax,
                           float* t_out, uint32_t* boundary_out);

/* ---- event server (continuous batching) ----------------------------------------------------------------------
 * The reference simulates one event per synchronous call (G4CXOpticks::simulate, g4cx/G4CXOpticks.cc:466-486;
 * its service layer CSGOptiX/CSGOptiXService.h answers one request at a time).  The server replaces that call for
 * multi-threaded producers: gbo_server_submit copies an event's gensteps (and input photons) and returns a ticket
 * at once (thread-safe); a worker thread packs waiting events into one simulate launch, runs up to `slots` launches
 * at once on separate streams, admits events while the launches' device buffers fit hbm_budget_bytes, and keeps
 * each finished event's hits on the host until gbo_server_release.  An event above max_batch_photon runs as
 * genstep-aligned pieces over several launches (as OPTICKS_MAX_SLOT slices an event in the reference,
 * qudarap/QSim.cc:481-529).  Results equal those of gbo_simulate for the same event id. */
typedef struct gbo_server gbo_server;
typedef struct gbo_server_config {
    int32_t slots;                  /* launches in flight at once (1..8, 2) */
    int32_t max_batch_events;       /* events per launch (4096) */
    int64_t max_batch_photon;       /* photons per launch (64M); also bounded by the budget; larger events are sliced */
    int64_t hbm_budget_bytes;       /* device memory the server's launches may hold (120 GB) */
    int64_t min_batch_photon;       /* while a launch is in flight, start another only once this many photons wait (2M) */
    int32_t use_graph;              /* 1: each batch's copies and kernels go out as one CUDA graph, captured from the
                                       stream and applied to the slot's executable graph by update (1) */
    int32_t big_exclusive;          /* 1: while a big batch's kernels run (an event of at least target_batch_photon),
                                       no other batch starts, so the big event keeps the whole GPU; 0: small batches
                                       may start beside it once min_batch_photon photons wait */
    int64_t target_batch_photon;    /* a batch stops taking events once it holds this many photons (4M): enough to
                                       fill the GPU, small enough that small events do not wait on a long launch */
    int64_t max_wait_us;            /* while a launch is in flight, waiting events start anyway once the oldest has
                                       waited this long, even below min_batch_photon (1000 us; 0: no limit) */
} gbo_server_config;
typedef struct gbo_server_stats {
    int64_t events_submitted, events_done, batches, photons, max_batch_photon;
    int64_t graph_launches, graph_instantiations;   /* instantiations: first batch of a slot, or topology change */
} gbo_server_stats;

int  gbo_server_config_default(gbo_server_config* cfg);
int  gbo_server_create(gbo_engine* e, const gbo_server_config* cfg, gbo_server** out);
int  gbo_server_submit(gbo_server* s, int32_t event_id, const gbo_quad6* gs, int64_t num_gs,
                       const gbo_sphoton* input_photon, int64_t num_input_photon, uint64_t* ticket);
int  gbo_server_wait(gbo_server* s, uint64_t ticket, int64_t timeout_us);          /* <0 : wait without limit */
int  gbo_server_event_info(gbo_server* s, uint64_t ticket, int64_t* num_photon, int64_t* num_hit, double* latency_s);
int  gbo_server_copy_hits(gbo_server* s, uint64_t ticket, gbo_sphoton* dst, int64_t offset, int64_t count);
int  gbo_server_release(gbo_server* s, uint64_t ticket);
int  gbo_server_get_stats(gbo_server* s, gbo_server_stats* out);
void gbo_server_destroy(gbo_server* s);

/* ---- event API on the engine handle --------------------------------------------------------------------------
 * The event server through the engine: the first submission starts a server with gbo_server_config_default that
 * the engine owns (gbo_engine_destroy stops it).  These are the submission / wait / hit-download / release calls a
 * threaded caller binds in place of SEvt::AddGenstep + G4CXOpticks::simulate + SEvt::GetNumHit / getHit +
 * G4CXOpticks::reset (sysrap/SEvt.hh:487, g4cx/G4CXOpticks.hh:95-96, sysrap/SEvt.cc:2050, :4991).  Submission is
 * thread-safe, copies its input and returns at once; timeouts are in nanoseconds (< 0: no limit). */
typedef uint64_t gbo_ticket;
int     gbo_event_submit(gbo_engine* e, const gbo_quad6* gs, size_t num_gs, uint32_t event_id, gbo_ticket* ticket);
int     gbo_event_submit_photons(gbo_engine* e, const gbo_quad6* gs, size_t num_gs, const gbo_sphoton* input_photon,
                                 size_t num_input_photon, uint32_t event_id, gbo_ticket* ticket);
int     gbo_event_wait(gbo_engine* e, gbo_ticket ticket, int64_t timeout_ns);       /* GBO_ERR_TIMEOUT: in flight */
int64_t gbo_event_num_hits(gbo_engine* e, gbo_ticket ticket);                       /* < 0: error (not done, unknown) */
int     gbo_event_copy_hits(gbo_engine* e, gbo_ticket ticket, gbo_sphoton* dst, size_t n);   /* the first n hits */
int     gbo_event_release(gbo_engine* e, gbo_ticket ticket);

/* The geometry handle of the drop-in contract is the engine (geometry uploaded to one GPU with its tables):
 * gbo_geometry_create = gbo_engine_create with gbo_config_default (the OPTICKS_* environment applied) on device 0. */
typedef struct gbo_engine gbo_geometry;
int  gbo_geometry_create(const gbo_geometry_desc* g, gbo_geometry** out);
void gbo_geometry_destroy(gbo_geometry* g);

/* gbo_simulate_noalloc : has no counterpart in the reference.  One event like gbo_simulate_device, for callers
 * that may not allocate device memory while events run (memory reserved up front by another runtime, or event
 * threads on which cudaMalloc/cudaFree must not be called because they synchronise the device).  Gensteps
 * (d_gs), optional input photons and the hit buffer (d_hits, room for hit_capacity hits) are the caller's device
 * memory; hits come back in photon order and *num_hit receives their number.  Everything else lives in one fixed
 * device array of gbo_noalloc_scratch_bytes() bytes (about 9.3 MB) that each GPU loading the library keeps until
 * the process exits; no allocating call is made.  Limits per call: 32768 gensteps, 4194304 photons, 131072 hits;
 * above them the call returns GBO_ERR_CAPACITY (for hits, *num_hit still reports the count).  The first call on a
 * device looks up the array's device address, so make it before any stream capture.  Calls share the array and
 * keep the previous call's contents: two calls in flight at the same time on one GPU race and corrupt each other,
 * so serialise them.  The call is synchronous on cuda_stream (NULL: the engine's stream). */
int64_t     gbo_noalloc_scratch_bytes(void);
int         gbo_simulate_noalloc(gbo_engine* e, int32_t event_id, const void* d_gs, int64_t num_gs,
                                 const void* d_input_photon, int64_t num_input_photon, gbo_sphoton* d_hits,
                                 int64_t hit_capacity, int64_t* num_hit, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* GBOPTICKS_H */
