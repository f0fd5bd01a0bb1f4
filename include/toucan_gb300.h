/* C ABI of the GB300 Toucan netlist simulator.
 *
 * Every entry point returns an int status: TGS_OK (0) or a negative TGS_ERR_*
 * code, with a message retrievable through tgs_last_error() (thread local).
 * Plain pointers and sizes only; no C++ or CUDA types cross this boundary.
 *
 * The reference runtime (ucsc-vama/toucanGPURT) keeps one simulator as
 * process-global device state (src/SimEval.cu:190-215) behind the C++ class
 * toucanGPUSim::ToucanSimulator (include/ToucanGPUSim.h:10-74).  Here each
 * simulator is a handle; the C++ class of the same name (ToucanGPUSim.h in
 * this directory) wraps one handle.  Each declaration names the reference
 * function it replaces.
 *
 * Value model (shared with the reference): every signal is a 4-bit nibble
 * stored in one byte; registers and memories are byte arrays (regPool,
 * memPool) addressed by nibble id.  A "stream" is one independent copy of
 * the design state driven by its own stimulus; the reference runs exactly
 * one stream, this library runs many at once.
 */
#ifndef TOUCAN_GB300_H
#define TOUCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TGS_OK = 0,
  TGS_ERR_ARG = -1,            /* bad argument (null handle, size mismatch...) */
  TGS_ERR_IO = -2,             /* file cannot be opened / read / written */
  TGS_ERR_FORMAT = -3,         /* design or symbol stream malformed or truncated */
  TGS_ERR_INVALID_DESIGN = -4, /* design violates a rule the evaluator relies on */
  TGS_ERR_CUDA = -5,           /* CUDA runtime error */
  TGS_ERR_NO_DEVICE = -6,      /* no usable GPU / unsupported compute capability */
  TGS_ERR_RESOURCES = -7,      /* shared memory, occupancy or co-residency too small */
  TGS_ERR_TIMEOUT = -8,        /* a device-side barrier wait ran out of its budget */
  TGS_ERR_STATE = -9,          /* call out of order (e.g. eval before init) */
  TGS_ERR_NOT_FOUND = -10,     /* unknown register / signal name */
  TGS_ERR_RANGE = -11,         /* value or size out of range */
  TGS_ERR_DEVICE_FAULT = -12   /* device-side check failed (address out of range...) */
};

typedef struct tgs_sim tgs_sim;

/* Message of the last failing call on this thread ("" if none). */
const char *tgs_last_error(void);
/* Library version string. */
const char *tgs_version(void);

/* ---- lifetime --------------------------------------------------------- */
int tgs_create(tgs_sim **out);
/* Frees all device and host memory of the handle.  The reference's
 * ToucanSimulator::cleanup (src/ToucanSim.cu:302-304) frees nothing. */
int tgs_destroy(tgs_sim *h);

/* ---- tuning ----------------------------------------------------------- */
typedef struct tgs_options {
  uint32_t n_streams;        /* independent design copies (default 1) */
  uint32_t warps_per_block;  /* 1 to 32; 0 = the most common exec-level width of the design (6..16) */
  uint32_t groups_per_item;  /* 8-stream groups one block evaluates together: 1, 2, 4 or 8; 0 = 4, halved
                                while a region would have fewer than two items per SM */
  uint32_t blocks_per_sm;    /* resident blocks per SM for the persistent grid (0 = max) */
  uint32_t schedule;         /* TGS_SCHED_GREEDY or TGS_SCHED_LEARNED */
  uint32_t mode;             /* TGS_MODE_PERSISTENT or TGS_MODE_GRAPH */
  uint32_t barrier_timeout_ms; /* budget of every device-side wait (default 2000) */
  uint32_t validate;         /* 1 = run the static design checks at init (default 1) */
  uint32_t resident_netlist; /* 0 (default): a block's exec levels stay in shared memory for the whole launch when
                                every block of the launch still fits on the GPU at once, else each level is staged
                                into shared memory while the previous one runs; 1: resident (TGS_ERR_RESOURCES when
                                it does not fit); 2: levels read from global memory; 3: staged */
  uint32_t value_pool;       /* 0: renumber value-pool slots by live range (default); 1: the design file's numbering.
                                Takes effect at the next tgs_init / tgs_init_from_memory */
  uint32_t capture_signals;  /* 1: record every signal of the symbol file each cycle (tgs_read_signal, VCD);
                                takes effect at the next tgs_init (tgs_enable_vcd also turns it on) */
  uint32_t lane_packing;     /* 0 (default): LUT micro-partitions of up to 16 lanes in one exec level are laid side
                                by side into 32-lane ones (same values, fewer warp passes); 1: the design file's
                                micro-partitions as they are.  Takes effect at the next tgs_init */
  uint32_t fast_luts;        /* 0 (default): LUT ops whose table row is a bitwise function of op1 and op2 (AND, OR,
                                XOR, ...) or a 0/1-select multiplexer -- checked entry by entry against the design's
                                table at load time -- are computed with word-wide logic for 8 streams at once, and
                                the ops of single-level LUT micro-partitions of an exec level are regrouped so that
                                such ops share warps; 1: every op by table lookup.  Takes effect at the next tgs_init,
                                for more than one stream (n_streams at init; one stream evaluates by lookup) */
  uint32_t mpart_lanes;      /* micro-partition size: LUTs a warp takes at once from an exec level's plan, 32
                                (0, the default), 64 or 128 -- 32-lane micro-partitions bundled by two or four when
                                warps are handed their share of a level (fewer, larger units per warp) */
  uint32_t levels_per_barrier; /* 1 (0, the default), 2 or 4: consecutive exec levels of a partition may run as one
                                block without a block barrier between them where every dependency among their
                                micro-partitions stays on one warp and the merged block is scheduled no longer than
                                the levels apart (chains of narrow cones); values are unchanged */
  uint32_t stage_words;      /* upper bound of a stage buffer in 32-bit words (0, the default: sized by the
                                library); exec levels larger than the buffers are read from global memory */
} tgs_options;

#define TGS_SCHED_GREEDY 0u
#define TGS_SCHED_LEARNED 1u
#define TGS_MODE_PERSISTENT 0u
#define TGS_MODE_GRAPH 1u

int tgs_default_options(tgs_options *opt);

/* Autotuner (no counterpart in the reference): times short runs of the loaded
 * design at the handle's stream count over groups_per_item x warps_per_block {4, 6, 8, 12, 16}
 * x blocks_per_sm x mode (x staging), then, with the fastest of those, over
 * micro-partition size (mpart_lanes {32, 64, 128}) x levels per barrier
 * {1, 2, 4}; keeps the fastest as the handle's options and resets the state
 * to the initial state. */
typedef struct tgs_tune_opts {
  uint32_t cycles;       /* timed cycles per trial (0 = 16) */
  uint32_t warmup;       /* untimed cycles per trial (0 = 2) */
  uint32_t modes;        /* bit 0: persistent, bit 1: graph (0 = both) */
  uint32_t try_unstaged; /* also try exec levels read from global memory */
  uint32_t reserved[4];
} tgs_tune_opts;

typedef struct tgs_tune_trial {
  uint32_t groups_per_item, warps_per_block, blocks_per_sm, mode;
  uint32_t staged;      /* exec levels: 1 staged per level, 2 resident for the launch, 0 read from global memory */
  uint32_t blocks;      /* grid size of the trial */
  float ms_per_cycle;   /* negative: the configuration does not fit */
  uint32_t mpart_lanes, levels_per_barrier;
} tgs_tune_trial;

/* trials (optional, max_trials entries) receives every trial; best receives the winner */
int tgs_autotune(tgs_sim *h, const tgs_tune_opts *opts, tgs_tune_trial *trials, uint32_t max_trials,
                 uint32_t *n_trials, tgs_tune_trial *best);
/* Takes effect at the next tgs_init / tgs_init_from_memory; n_streams and the
 * schedule may also be changed after init (state is reset to the initial state). */
int tgs_set_options(tgs_sim *h, const tgs_options *opt);
int tgs_get_options(const tgs_sim *h, tgs_options *opt);

/* ---- ToucanSimulator API ---------------------------------------------- */
/* ToucanSimulator::init (src/ToucanSim.cu:102-204): load the design and
 * symbol files, Init(), optionally Randomize(seed 0), upload.  0 on success,
 * TGS_ERR_IO where the reference returns -1 for a missing file. */
int tgs_init(tgs_sim *h, int gpu_id, const char *design_path, const char *symbol_path, int randomize,
             int enable_print);
/* Same from in-memory serialized design / symbol streams. */
int tgs_init_from_memory(tgs_sim *h, int gpu_id, const void *design, size_t design_bytes, const void *symbols,
                         size_t symbol_bytes, int randomize, int enable_print);

/* ToucanSimulator::eval (src/ToucanSim.cu:206-230): one cycle of every
 * stream; *stop = sticky stop flag of stream 0 (any stream in batched use). */
int tgs_eval(tgs_sim *h, int *stop);
/* ToucanSimulator::eval_free_running (src/ToucanSim.cu:232-267): `cycles`
 * cycles in one persistent launch; like the reference it does not stop early. */
int tgs_eval_free_running(tgs_sim *h, uint32_t cycles, int *stop);
/* Free running with the early exit the reference leaves commented out
 * (src/SimEval.cu:990-992): a stream that executes a stop op freezes after
 * that cycle and the launch ends once every stream stopped, or after
 * max_cycles.  *cycles_run = cycles executed (added to cycle_cnt and
 * realCycles).  No counterpart in the reference. */
int tgs_eval_until_stop(tgs_sim *h, uint32_t max_cycles, int *stop, uint32_t *cycles_run);

/* ToucanSimulator::setRegister / readRegister (src/ToucanSim.cu:271-289,
 * src/SimEval.cu:1058-1081): value split into nibbles, most significant
 * first, at most 16 nibbles.  TGS_ERR_RANGE when the value is wider than the
 * register (the reference asserts).  Stream 0. */
int tgs_set_register(tgs_sim *h, const char *name, uint64_t value);
int tgs_read_register(tgs_sim *h, const char *name, uint64_t *value);
/* Per-stream variants. */
int tgs_set_register_stream(tgs_sim *h, uint32_t stream, const char *name, uint64_t value);
int tgs_read_register_stream(tgs_sim *h, uint32_t stream, const char *name, uint64_t *value);
/* read_reg_from_gpu for many registers (src/SimEval.cu:1058-1069,
 * src/ToucanSim.cu:280-289): values[i] = register names[i] of `stream`,
 * most significant nibble first.  One gather kernel and one device-to-host
 * copy per call (the reference issues one blocking copy per nibble). */
int tgs_read_registers(tgs_sim *h, uint32_t stream, const char *const *names, uint32_t n, uint64_t *values);

/* ToucanSimulator::readSignal (src/ToucanSim.cu:291-300; unimplemented in
 * the reference, which returns UINT64_MAX): the value of a signal of the
 * symbol file's signalDebugInfo in the last evaluated cycle.  A signal is a
 * list of (partition, value-pool slot, width) sections, most significant
 * first (the order of the reference's VCD writer, unsupport/SimVCD.cpp);
 * each section's value is the slot's nibble after the partition's exec
 * levels.  Needs options.capture_signals (else TGS_ERR_STATE); at most 64
 * bits (TGS_ERR_RANGE).  A section whose slot the partition never writes
 * has no defined value. */
int tgs_read_signal(tgs_sim *h, const char *name, uint64_t *value);
int tgs_read_signal_stream(tgs_sim *h, uint32_t stream, const char *name, uint64_t *value);
/* ToucanSimulator::enableVCDDump (unsupport/SimVCD.cpp:99-241, not built by
 * the reference): writes a VCD file of every signal of stream 0, one time
 * step per tgs_eval (#c = the values of cycle c) and one per
 * tgs_eval_free_running / tgs_eval_until_stop (its last cycle).  Turns signal
 * capture on, which needs a new device image: allowed before the first
 * cycle only (TGS_ERR_STATE afterwards) unless capture_signals was set at
 * init. */
int tgs_enable_vcd(tgs_sim *h, const char *path);

/* get_real_cycles / setEnablePrint / get_eval_done (src/SimEval.cu:1083-1097) */
int tgs_get_real_cycles(tgs_sim *h, uint32_t *cycles);
int tgs_get_cycle_cnt(tgs_sim *h, uint64_t *cycles);
int tgs_set_enable_print(tgs_sim *h, int enable);
int tgs_get_eval_done(tgs_sim *h, int *stop);

/* copy_profile_data (src/SimEval.cu:1101-1104): per-partition mean clock64
 * ticks, "useful" (partition work) and "total" (including barrier wait),
 * over cycles [PROFILE_START_CYCLE, +PROFILE_COLLECT_CYCLE) of the last
 * free-running launch.  Here always available (no rebuild needed). */
int tgs_copy_profile_data(tgs_sim *h, int64_t *useful_ticks, int64_t *total_ticks, size_t count);

/* ---- bulk state access (new) ------------------------------------------ */
int tgs_get_pool_sizes(const tgs_sim *h, uint32_t *reg_pool, uint32_t *mem_pool, uint32_t *exchange_pool);
/* Full regPool / memPool of one stream (reference byte layout). */
int tgs_read_reg_pool(tgs_sim *h, uint32_t stream, uint8_t *out, size_t bytes);
int tgs_write_reg_pool(tgs_sim *h, uint32_t stream, const uint8_t *in, size_t bytes);
int tgs_read_mem_pool(tgs_sim *h, uint32_t stream, uint8_t *out, size_t bytes);
int tgs_write_mem_pool(tgs_sim *h, uint32_t stream, const uint8_t *in, size_t bytes);
/* Digests as defined for the oracle: sum over i of mix64((i << 8) | pool[i]). */
int tgs_state_digest(tgs_sim *h, uint32_t stream, uint64_t *reg_digest, uint64_t *mem_digest);
/* Reset every stream to the initial state (Init/Randomize result). */
int tgs_reset_state(tgs_sim *h);

/* Checkpoint (no counterpart in the reference): every stream's register and
 * memory pools, stop flags, stop cycles and rolling digests, plus the cycle
 * counters, written to a file in a layout independent of the launch options.
 * tgs_load_state restores it into a handle holding the same design (checked
 * by a fingerprint of the design's structure); the handle takes the file's
 * stream count.  A run continued after a load (eval, eval_free_running,
 * tgs_batch_run with TGS_BATCH_CONTINUE) gives the results of the run that
 * was never interrupted. */
int tgs_dump_state(tgs_sim *h, const char *path);
int tgs_load_state(tgs_sim *h, const char *path);

/* Same digest as tgs_state_digest, of caller-owned device memory, for
 * callers that cannot allocate device memory (an allocator that owns every
 * device byte, a frozen memory pool).  No counterpart in the reference.
 * pools: device pointer, pool i at pools + i * stride, `bytes` bytes each
 * (bytes < 4 GiB); digests: host array of n_pools results.  At most 4,096
 * pools per call (TGS_ERR_RANGE above that).  Allocates nothing: the
 * per-pool accumulators are a fixed 32 KiB device array inside the library,
 * present on every GPU that loads it until the process exits.  Every call
 * looks up that array's address in the current device's context (so a
 * context re-created by cudaDeviceReset is followed); the first call on a
 * device loads the library's device code there, so make it before any
 * stream capture.  Runs on the legacy default stream and waits for it: the
 * caller must first synchronise the stream or event that wrote the pools
 * when that stream does not synchronise with the legacy default stream (a
 * cudaStreamNonBlocking stream, or code built with per-thread default
 * streams), else the digests may read stale bytes.  All calls share the
 * one array, so calls that overlap on the GPU (other host threads) race. */
int tgs_pool_digests_noalloc(const uint8_t *pools, uint64_t stride, uint64_t bytes, uint32_t n_pools,
                             uint64_t *digests);

/* ---- batched stimulus runs (new) -------------------------------------- */
/* Stimulus: the listed register nibbles are rewritten before every cycle.
 *   seed_s = mix64(base_seed ^ s); h = mix64(seed_s ^ mix64((c << 32) | i))
 *   toggle[i] == 0: value = h & mask(bits[i]); else the value flips (xor
 *   mask) when (h >> 48) < toggle[i].  mix64 = splitmix64 finaliser. */
typedef struct tgs_stimulus {
  uint64_t base_seed;
  uint32_t n_inputs;
  const uint32_t *reg;     /* regPool nibble ids */
  const uint8_t *bits;     /* bit width of each input nibble (1..4) */
  const uint16_t *toggle;  /* NULL = all inputs uniform */
  /* Optional host table of input values, [cycle][input][stream] one nibble
   * per byte (written to the register nibble as is), covering the cycles of
   * this call (runs where every stream is resident and equally long);
   * replaces the seeded values.  Pinned memory (tgs_host_alloc) makes the
   * upload faster. */
  const uint8_t *table;
} tgs_stimulus;

#define TGS_BATCH_CYCLE_DIGESTS 1u /* fill cycle_digest[] */
#define TGS_BATCH_ROLLING 2u       /* fill rolling_digest[] */
#define TGS_BATCH_FINAL_STATE 4u   /* fill final_regs[] / final_mems[] */
#define TGS_BATCH_CONTINUE 8u      /* continue every stream from the previous call's state and cycle */
#define TGS_BATCH_STOP_EXIT 16u    /* a stream that executes a stop op ends after that cycle (registers,
                                      memories, digests freeze); resident streams: the launch ends once every
                                      stream stopped; queued streams: the stopped stream retires and its slot
                                      takes the next queued stream. */

typedef struct tgs_batch {
  uint32_t n_streams;       /* streams in the job (may exceed resident slots) */
  const uint32_t *cycles;   /* cycles per stream */
  const tgs_stimulus *stim; /* NULL = free running */
  uint32_t flags;
  uint32_t slots;           /* resident streams (rounded up to a multiple of 8, at most 4096 when streams
                               queue); 0 = total cycles / longest stream (clamped to 8..4096): queued
                               streams are admitted longest first */
} tgs_batch;

typedef struct tgs_batch_result {
  uint64_t *final_reg_digest; /* [n_streams] */
  uint64_t *final_mem_digest; /* [n_streams] */
  uint64_t *rolling_digest;   /* [n_streams]: roll = mix64(roll + digest(c)) */
  uint64_t *cycle_digest;     /* [n_streams * cycle_stride] */
  uint32_t cycle_stride;
  uint32_t *stop_cycle;       /* [n_streams], 0xFFFFFFFF = no stop */
  uint8_t *final_regs;        /* [n_streams * regPoolSize] */
  uint8_t *final_mems;        /* [n_streams * memPoolSize] */
  double device_ms;           /* time of the device work */
  uint64_t stream_cycles;     /* total simulated stream-cycles (stop exit: through each stop cycle) */
  uint32_t launches;          /* kernel launches issued */
} tgs_batch_result;

/* Runs every stream of the job from the initial state.  With equal lengths
 * and all streams resident, one launch runs them side by side.  Otherwise
 * the streams are queued, longest first, onto `slots` resident slots:
 * a slot whose stream finished is retired and refilled in place by the next
 * queued stream inside the same launch (final digests, rolling
 * digests, per-cycle digests and stop cycles are reported per job stream;
 * final_regs / final_mems are not available in that form). */
int tgs_batch_run(tgs_sim *h, const tgs_batch *job, tgs_batch_result *res);

/* Page-locked host memory for stimulus tables and results. */
int tgs_host_alloc(size_t bytes, void **out);
int tgs_host_free(void *p);

/* Releases everything the library holds on `device` (cudaDeviceReset
 * through the library's own CUDA runtime: the device's primary context is
 * destroyed with every allocation in it, the caller's included, and
 * re-created on the next use).  Destroy every handle on the device first;
 * page-locked buffers from tgs_host_alloc are freed with the context. */
int tgs_device_reset(int device);

/* ---- design statistics and launch shape (new) ------------------------- */
typedef struct tgs_design_stats {
  uint64_t lut_ops;          /* table lookups (lutIndex != 0) */
  uint64_t nop_ops;          /* moves (lutIndex == 0) */
  uint64_t writeback_ops;    /* micro-partition write-back lanes */
  uint64_t l0_reg_reads, l0_exg_reads;
  uint64_t reg_copy_slots, exg_copy_slots; /* nibbles moved by the block copies */
  uint64_t mem_read_ops, mem_write_ops, vec_ops, vec_read_ops, print_ops, stop_ops;
  uint64_t op_slots;         /* every op slot, 32-bit words of instruction per cycle */
  uint32_t partitions, mparts, max_value_pool, max_exec_levels;
  uint32_t blocks, threads, groups_per_item, streams_per_word;
  uint64_t block_barriers, exec_levels;   /* block barriers kept / exec levels, all partitions */
  double makespan[2];        /* scheduled cost of the slowest block per region */
  uint32_t smem_per_block;   /* dynamic shared memory of a block: table, stage buffers, value pool */
  uint32_t stage_words;      /* words of one exec-level stage buffer (0: levels resident or read from global memory) */
  uint32_t resident_words;   /* words of a block's resident exec levels (0: staged or read from global memory) */
  uint32_t fused_levels;     /* exec levels merged into the block before them (levels_per_barrier > 1) */
  uint32_t reserved[4];
} tgs_design_stats;
int tgs_get_design_stats(const tgs_sim *h, tgs_design_stats *out);

/* ---- learned cost model of micro-partitions (new) ----------------------- */
/* The scheduler (options.schedule = TGS_SCHED_LEARNED) balances warps and
 * blocks on a cost predicted by a 16-64-64-1 FP32 MLP from 16 structural
 * features of each micro-partition, trained with Adam on clock64 timings the
 * cycle kernel records; gate count (TGS_SCHED_GREEDY) is the fallback.
 * Values never depend on the schedule. */
typedef struct tgs_train_opts {
  uint32_t epochs;   /* default 30 */
  uint32_t batch;    /* default 1024 */
  float lr;          /* default 2e-3 */
  uint64_t seed;
  float val_frac;    /* held-out fraction for the report (<= 0.5) */
  uint32_t reserved[4];
} tgs_train_opts;

typedef struct tgs_train_report {
  float train_mse, val_mse;  /* standardised log-cycle space */
  float val_corr;            /* correlation of predicted and measured log cycles (held out) */
  float gate_corr;           /* same for log gate count (the greedy cost) */
  uint32_t samples, epochs;
  double train_ms;
  uint32_t reserved[4];
} tgs_train_report;

int tgs_num_mparts(tgs_sim *h, uint32_t *n);
/* features[id * 16 + f] of every micro-partition (id = design order) */
int tgs_mpart_features(tgs_sim *h, float *features, uint32_t n);
/* runs `cycles` cycles of every stream with per-micro-partition clock64
 * timing; mean_cycles[id] = mean cycles of one evaluation */
int tgs_profile_mparts(tgs_sim *h, uint32_t cycles, float *mean_cycles, uint32_t n);
/* trains the handle's cost model (rebuilds a learned schedule) */
int tgs_cost_model_train(tgs_sim *h, const float *features, const float *cycles, uint32_t n, const tgs_train_opts *opts,
                         tgs_train_report *report);
/* get (set = 0) or set (set = 1) the 5,313 parameters + (mean, std) of log cycles */
int tgs_cost_model_state(tgs_sim *h, float *state, size_t n, int set);
/* the network's kernels on host buffers: outputs for n feature rows, and the
 * mean-squared-error gradient (for checks against a CPU reference) */
int tgs_mlp_forward(const float *params, const float *X, uint32_t n, float *out);
int tgs_mlp_grad(const float *params, const float *X, const float *y, uint32_t n, float *grad, float *loss);

/* ---- synthetic designs (new; the reference ships no design or compiler) */
typedef struct tgs_gen_config {
  uint64_t seed;
  uint64_t n_lut;          /* LUT ops with a table lookup */
  uint32_t levels;         /* logic levels per cycle (split over the two regions) */
  uint32_t operands;       /* 2 (op0 = 0) or 3 nibble operands per LUT */
  uint32_t ff_bits;        /* flip-flop bits (4 per register nibble) */
  uint32_t pi_bits;        /* primary-input bits (register nibbles rewritten by the stimulus) */
  uint32_t reset_inputs;   /* extra 1-bit primary inputs */
  uint32_t n_mems, mem_depth, mem_width, mem_read_ports, mem_write_ports;
  uint32_t mem_multi_writer; /* 1: index = memBase + (addr << 2) */
  uint32_t n_vec_ops, vec_nibbles;
  uint32_t palette_pct;    /* % of LUTs using AND/OR/XOR/MUX windows */
  float fanout_alpha;      /* power-law exponent of operand popularity (0 = uniform) */
  uint32_t max_fanout;
  uint32_t luts_per_part;  /* partition size target */
  uint32_t mpart_width;    /* lanes per micro-partition level (<= 32) */
  uint32_t cone_depth;     /* logic levels per micro-partition (1 = top level only) */
  uint32_t mixed;          /* 1: heterogeneous regions (datapath / control / memory / fan-out) */
  uint32_t with_stop;      /* add a stop op (and print): 1 enabled by a design value (fires early),
                              2 enabled when a design value equals a constant (about 1 cycle in 16) */
  uint32_t signals;        /* internal signals listed in the symbol file (signalDebugInfo), 0 = none */
  uint32_t reserved[5];
} tgs_gen_config;

typedef struct tgs_gen_info {
  uint64_t lut_ops, nop_ops, mparts, partitions;
  uint64_t mem_read_ops, mem_write_ops, vec_ops, l0_ops;
  uint32_t reg_pool, mem_pool, exchange_pool, max_value_pool;
  uint32_t n_pi_nibbles;   /* primary-input nibble ids are listed by tgs_gen_inputs */
  uint32_t reserved[7];
} tgs_gen_info;

int tgs_default_gen_config(tgs_gen_config *cfg);
/* Generates a design, writes the design and symbol files (reference format). */
int tgs_generate(const tgs_gen_config *cfg, const char *design_path, const char *symbol_path, tgs_gen_info *info);
/* Primary-input nibble ids and widths of a design generated with cfg
 * (ids: [n], bits: [n]; n from tgs_gen_info.n_pi_nibbles). */
int tgs_gen_inputs(const tgs_gen_config *cfg, uint32_t *ids, uint8_t *bits, uint32_t n);

/* Host-only file utilities (no GPU needed).  tgs_resave_* load a file with
 * this library's loader and write it back with its serializer (byte for byte
 * the reference format).  tgs_initial_state: Init() and optionally
 * Randomize(0) (reference src/SimInit.cpp:16-64) into caller buffers of
 * regPoolSize / memPoolSize bytes. */
int tgs_resave_design(const char *in_path, const char *out_path);
int tgs_resave_symbols(const char *in_path, const char *out_path);
int tgs_initial_state(const char *design_path, const char *symbol_path, int randomize, uint8_t *regs, size_t reg_bytes,
                      uint8_t *mems, size_t mem_bytes);

/* Static checks of a design file: the rules that make a design's values
 * independent of the schedule (def-before-use, no same-level slot conflicts,
 * word-aligned block copies, table bounds, nibble-valued tables). */
int tgs_validate_file(const char *design_path, const char *symbol_path, uint64_t *lut_ops);

/* Writes the design with every partition's value-pool slots renumbered by
 * live range, the relabelling tgs_init applies to the device image when the
 * value_pool option is 0 (no counterpart in the reference).  max_before /
 * max_after (optional): the largest valuePoolSize before and after. */
int tgs_compact_design(const char *in_path, const char *out_path, uint32_t *max_before, uint32_t *max_after);
/* Writes the design with the lane packing tgs_init applies by default
 * (options.lane_packing = 0): in every exec level, LUT micro-partitions of up
 * to 16 lanes laid side by side into 32-lane ones, each member's lane
 * references shifted to its lanes and shallower members carried through the
 * extra middle levels by moves of their own lanes.  The result is a valid
 * design of the same format that computes the same values (so any evaluator,
 * the CPU oracle included, can check the packing).  No counterpart in the
 * reference.  mparts_before / mparts_after: micro-partitions in all exec
 * levels (either may be NULL). */
int tgs_pack_design(const char *in_path, const char *out_path, uint32_t *mparts_before, uint32_t *mparts_after);
/* Writes the design with the micro-partition transforms tgs_init applies by
 * default: lane packing (as tgs_pack_design) and then, with fast_luts, the
 * regrouping of every exec level's single-level LUT micro-partitions by kind
 * (ops with a word-wide form first, then ops that need table lookups; see
 * tgs_options.fast_luts).  Same format, same values: any evaluator, the CPU
 * oracle included, can check it.  No counterpart in the reference.  stats
 * (optional) receives the micro-partition counts and the LUT ops (lutIndex
 * != 0) that the device image evaluates word-wide. */
typedef struct tgs_repack_stats {
  uint64_t mparts_before, mparts_after;
  uint64_t lut_ops;        /* LUT ops with lutIndex != 0 */
  uint64_t fast_lut_ops;   /* of which evaluated with word-wide logic */
  uint64_t fast_mparts;    /* micro-partitions whose top level is word-wide */
  uint64_t exec_levels;    /* exec levels of all partitions */
  uint64_t reserved[2];
} tgs_repack_stats;
int tgs_repack_design(const char *in_path, const char *out_path, int lane_packing, int fast_luts,
                      tgs_repack_stats *stats);

/* The exec-level schedule tgs_init would build for a design, computed on the
 * host only (no GPU): the device image (renumbered value pool, lane packing
 * unless lane_packing = 1, word-wide ops when fast_luts = 0 and more than one
 * stream) and the gate-count schedule for `warps` warps per block and
 * `groups` stream groups per item, with the schedule knobs mpart_lanes and
 * levels_per_barrier (0 = defaults), for one block.  For checking and
 * comparing schedules; tgs_get_design_stats reports the live one. */
typedef struct tgs_schedule_stats {
  uint64_t exec_levels;      /* exec levels of all partitions */
  uint64_t blocks;           /* level blocks emitted (exec levels less the fused ones) */
  uint64_t barriers;         /* level blocks that start with a block barrier */
  uint64_t fused_levels;     /* exec levels merged into the block before them */
  uint64_t schedule_words;   /* words of all level blocks */
  uint32_t max_level_words;  /* largest level block */
  uint32_t reserved0;
  double makespan;           /* sum over level blocks of the most loaded warp's gate count */
  double work;               /* sum of all units' gate counts */
  double level_bound;        /* sum over level blocks of max(work / warps, largest unit): no schedule is shorter */
  double list_bound;         /* sum over level blocks of work / warps + largest unit: a list schedule of
                                single units (mpart_lanes 32, no fused levels) is not longer */
  uint64_t reserved[3];
} tgs_schedule_stats;
int tgs_plan_schedule(const char *design_path, uint32_t warps, uint32_t groups, uint32_t mpart_lanes,
                      uint32_t levels_per_barrier, int lane_packing, int fast_luts, uint32_t n_streams,
                      tgs_schedule_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
