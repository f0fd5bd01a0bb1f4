/* CPU oracle for the Toucan per-cycle netlist evaluation.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * entry point and the CPU-baseline leg of bench.py may load it; the product
 * (toucangpurt_gb300) never links, loads or calls it.
 *
 * It restates the reference evaluator (src/SimEval.cu:304-995 and
 * src/SimInit.cpp:16-64 of ucsc-vama/toucanGPURT) op by op on the CPU, with
 * its own design-file parser, and adds the multi-stream stimulus and digest
 * definitions the GPU path is compared on. */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_design orc_design;

/* Stimulus: each listed register nibble is rewritten before every cycle.
 *   seed_s  = mix64(base_seed ^ s)                 (per stream s)
 *   h       = mix64(seed_s ^ mix64((c << 32) | i)) (cycle c, input i)
 *   toggle[i] == 0 : value = h & mask(bits[i])
 *   toggle[i] >  0 : value ^= mask(bits[i]) when (h >> 48) < toggle[i]
 * mix64 is the splitmix64 finaliser (Steele, Lea, Flood 2014). */
typedef struct orc_stimulus {
  uint64_t base_seed;
  uint32_t n_inputs;
  const uint32_t *reg;     /* regPool nibble id */
  const uint8_t *bits;     /* 1..4 */
  const uint16_t *toggle;  /* may be NULL: all uniform */
} orc_stimulus;

typedef struct orc_result {
  uint64_t *final_reg_digest;  /* [n_streams] or NULL */
  uint64_t *final_mem_digest;  /* [n_streams] or NULL */
  uint64_t *rolling_digest;    /* [n_streams] or NULL: fold of per-cycle reg digests */
  uint64_t *cycle_digest;      /* [n_streams * cycle_stride] or NULL */
  uint32_t cycle_stride;
  uint32_t *stop_cycle;        /* [n_streams] or NULL: first cycle a stop op fired, 0xFFFFFFFF none */
  uint8_t *final_regs;         /* [n_streams * regPoolSize] or NULL */
  uint8_t *final_mems;         /* [n_streams * memPoolSize] or NULL */
} orc_result;

orc_design *orc_load(const char *design_path, const char *symbol_path, int randomize, char *err, size_t errlen);
void orc_free(orc_design *d);
uint32_t orc_reg_pool_size(const orc_design *d);
uint32_t orc_mem_pool_size(const orc_design *d);
uint32_t orc_num_parts(const orc_design *d);
uint64_t orc_num_lut_ops(const orc_design *d); /* LUT ops with lutIndex != 0 */
const uint8_t *orc_initial_regs(const orc_design *d);
const uint8_t *orc_initial_mems(const orc_design *d);

/* Run n_streams independent streams from the design's initial state.
 * cycles[s] cycles each; stim may be NULL (free running).  threads <= 0 uses
 * all hardware threads.  Returns 0, or -1 with a message in err (e.g. a
 * memory address out of range). */
int orc_run(const orc_design *d, uint32_t n_streams, const uint32_t *cycles, const orc_stimulus *stim,
            orc_result *res, int threads, char *err, size_t errlen);

/* Reference-style single-stream stepping (eval() / setRegister flow). */
typedef struct orc_state orc_state;
orc_state *orc_state_new(const orc_design *d);
void orc_state_free(orc_state *s);
int orc_state_eval(orc_state *s, uint32_t cycles, int *stop, char *err, size_t errlen);
uint8_t *orc_state_regs(orc_state *s);
uint8_t *orc_state_mems(orc_state *s);
/* Signal probes: slot slots[i] of partition parts[i], recorded after the
 * partition's exec levels every cycle; values of the last evaluated cycle. */
int orc_state_set_probes(orc_state *s, const uint32_t *parts, const uint32_t *slots, uint32_t n);
const uint8_t *orc_state_probe_values(const orc_state *s);
uint64_t orc_digest(const uint8_t *pool, size_t n);
uint64_t orc_mix64(uint64_t x);

#ifdef __cplusplus
}
#endif
