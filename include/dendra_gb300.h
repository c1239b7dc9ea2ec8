/*
 * dendra_gb300 — C ABI of the GB300 (sm_103a) cable-update library.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t
 * passed as `void*` (NULL = legacy default stream).  No entry point
 * allocates device memory unless its comment says so; callers own every
 * buffer.  Floating-point buffers are float32 or float64 as selected by the
 * `dtype` argument (DGB_F32 / DGB_F64); index buffers are int32/int64 as
 * declared.  Every function returns 0 on success or a negative DGB_E* code;
 * `dgb_last_error()` gives a message for the last failure on the calling
 * thread.
 *
 * Reference interfaces replaced (paths are relative to the Dendra source
 * tree, v0.30.1):
 *   dgb_tridiag_solve         dendra/models/integrators/triton/t_kernel_thomas.py:218-232
 *                             (thomas_solve_cuda_t) and pcr_kernel_thomas.py:199-226
 *                             (pcr_solve_cuda_t); solver callable selected in
 *                             integrators/implicit.py:364-440, called at :647
 *   dgb_tridiag_solve_transpose  ThomasSolve.backward, t_kernel_thomas.py:147-189
 *   dgb_cable_run             one Population.run over an unbranched HH cable
 *                             population: models/core.py:4555-4628 driving
 *                             integrators/core.py:769-834 and
 *                             integrators/implicit.py:569-664
 *   dgb_cable_assemble        the eager per-step assembly of the same update
 *                             (mechanism advance + membrane frame + RHS),
 *                             integrators/core.py:769-834, implicit.py:569-646
 */
#ifndef DENDRA_GB300_H
#define DENDRA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* dtype selectors */
#define DGB_F32 0
#define DGB_F64 1

/* tridiagonal methods */
#define DGB_THOMAS 0
#define DGB_PCR 1

/* error codes */
#define DGB_OK 0
#define DGB_EINVAL -1   /* bad argument (shape, dtype, null pointer) */
#define DGB_ECUDA -2    /* CUDA launch or runtime failure */
#define DGB_ETIMEOUT -3 /* a bounded device-side wait gave up */
#define DGB_ERANGE -4   /* a size beyond a documented maximum */

/* Library version string. */
const char* dgb_version(void);

/* Message for the last failure on the calling host thread ("" if none). */
const char* dgb_last_error(void);

/* sizeof(dgb_cable_args) as compiled (for foreign-language mirrors). */
size_t dgb_cable_args_size(void);

/*
 * Batched tridiagonal solve, B independent systems of size K.
 *   a: (B, K-1) sub-diagonal,  b: (B, K) diagonal,
 *   c: (B, K-1) super-diagonal, d: (B, K) right-hand side,
 *   x: (B, K) solution (may alias d).
 * Row-major contiguous.  method = DGB_THOMAS or DGB_PCR; both run the same
 * register-resident chunked solve (sequential elimination inside each lane's
 * chunk, parallel cyclic reduction across lanes by warp shuffles); the method
 * selects the lanes per system (THOMAS: the autotuned split, PCR: the widest
 * split).  Replaces thomas_solve_cuda_t / pcr_solve_cuda_t.
 */
int dgb_tridiag_solve(int dtype, int method, int64_t B, int64_t K,
                      const void* a, const void* b, const void* c,
                      const void* d, void* x, void* stream);

/*
 * As dgb_tridiag_solve with an explicit lanes-per-system split (4, 8, 16 or
 * 32; 0 = default), the knob the autotuner sweeps.
 */
int dgb_tridiag_solve_lanes(int dtype, int64_t B, int64_t K, const void* a,
                            const void* b, const void* c, const void* d,
                            void* x, int32_t lanes, void* stream);

/*
 * Solve the transposed systems A^T y = g for the same bands (adjoint of
 * dgb_tridiag_solve): the transpose has sub-diagonal c and super-diagonal a.
 * Replaces the transpose solve inside ThomasSolve.backward.
 */
int dgb_tridiag_solve_transpose(int dtype, int64_t B, int64_t K,
                                const void* a, const void* b, const void* c,
                                const void* g, void* y, void* stream);

/*
 * Arguments of a multi-step unbranched Hodgkin–Huxley cable run.
 * All per-compartment arrays are packed cable after cable, with cable i
 * occupying [cable_ptr[i], cable_ptr[i+1]).  Per-cable arrays have n_cables
 * entries.  Optional pointers may be NULL.  Floating pointers use `dtype`.
 */
typedef struct dgb_cable_args {
  int32_t dtype;
  int32_t n_cables;
  int32_t n_steps;
  int32_t rec_every;        /* record every rec_every steps (>=1) */
  const int64_t* cable_ptr; /* [n_cables+1], device */
  const int32_t* order;     /* [n_cables] work order (largest first), device; NULL = identity */
  /* state, in/out */
  void* v;
  void* m;
  void* h;
  void* n;
  /* prepared workspace (integrators/implicit.py:484-522) */
  const void* g_right; /* g_edge(i,i+1)/C_i, 0 on the last compartment */
  const void* g_left;  /* g_edge(i-1,i)/C_i, 0 on the first compartment */
  const void* scale;   /* area/C */
  const void* cm_inv;  /* 1/C */
  const void* field;   /* extracellular lead field, mV per mA (NULL: no ve) */
  /* HH channel densities per compartment (S/cm^2) and leak reversal (mV) */
  const void* gnabar;
  const void* gkbar;
  const void* gl;
  const void* el;
  double ena, ek, q10;
  double dt_ms;   /* timestep in ms */
  double dt_s;    /* timestep in s, rounded in the state dtype */
  double t0_ms;   /* time origin */
  int64_t step0;  /* index of the first step: step s runs at t0_ms + (step0 + s) dt_ms */
  /* extracellular pulse per cable: ve = field * amp on [delay, delay+pw) */
  const void* ve_amp;
  const void* ve_delay;
  const void* ve_pw;
  /* intracellular current clamp per cable (mA) at local compartment in_idx */
  const int32_t* in_idx;
  const void* in_amp;
  const void* in_delay;
  const void* in_pw;
  /* recording: local compartment per cable (-1: none); trace is
     [n_cables][1 + n_steps/rec_every] in the state dtype */
  const int32_t* rec_idx;
  void* trace;
  /* spike detection: rising edge v >= spk_thr at local compartment spk_idx
     (-1: none); below latch in/out, counts and first crossing step out */
  const int32_t* spk_idx;
  double spk_thr;
  int32_t* spk_below;
  int32_t* spk_count;
  int32_t* spk_first;
  /* sizes known to the host: largest cable and total compartments */
  int32_t max_k;       /* max over cables of K */
  int32_t flags;       /* DGB_CABLE_* bits */
  int64_t n_comp;      /* cable_ptr[n_cables] */
  /* cable index of every compartment, int32[n_comp] (assembly kernel only) */
  const int32_t* comp_cable;
  /* scratch, int32[2] on the device (dgb_cable_run only): [0] work counter,
     [1] error bits after the run (0 = every cable advanced) */
  int32_t* scratch;
} dgb_cable_args;

/* dgb_cable_args.flags bits.
   UNIFORM_CHANNELS: gnabar, gkbar, gl, el are constant within each cable.
   UNIFORM_GEOMETRY: g_right (all but the last compartment), g_left (all but
     the first) and scale are constant within each cable.
   The kernel then reads those values once per cable (exactly the same values).
   FAST_MATH (float32 only): approximate reciprocals and shared exponentials in
     the gate advance and the solve; the results stay within the float32
     tolerance of the exact path (1e-3 mV against a float64 run). */
#define DGB_CABLE_UNIFORM_CHANNELS 1
#define DGB_CABLE_UNIFORM_GEOMETRY 2
#define DGB_CABLE_FAST_MATH 4

/*
 * Run n_steps backward-Euler + cnexp steps of every cable in one persistent
 * launch.  State stays in registers and shared memory for the whole run; only
 * the recorded trace and spike results are written during the run.
 * Replaces the per-step Population.run loop for an HH unbranched population.
 */
int dgb_cable_run(const dgb_cable_args* args, void* stream);

/*
 * One unfused step, first half: advance the gates and assemble the
 * tridiagonal system of every compartment (lower/main/upper/rhs) for the
 * state in args (v, m, h, n are read; m, h, n are written).  With
 * dgb_tridiag-style solve and dgb_cable_update it forms the plain per-step
 * path the persistent run is compared against.  `step` is the step index
 * used for the pulses.  Bands are packed like the state: lower/upper have a
 * zero at each cable's boundary row.
 */
int dgb_cable_assemble(const dgb_cable_args* args, int32_t step,
                       void* lower, void* main_diag, void* upper, void* rhs,
                       void* stream);

/*
 * Solve the packed ragged systems produced by dgb_cable_assemble and add the
 * increment to v (v += x).
 */
int dgb_cable_solve_update(const dgb_cable_args* args, const void* lower,
                           const void* main_diag, const void* upper,
                           const void* rhs, void* stream);

/*
 * Allocation-free unfused step: dgb_cable_assemble + dgb_cable_solve_update
 * with their band scratch in a 4 MiB array compiled into the library
 * (at most 262,144 float32 or 131,072 float64 compartments; larger
 * populations return DGB_ERANGE).  No counterpart in the reference: it
 * serves callers that cannot allocate device memory on their call path
 * (hosts that preallocate all GPU memory up front, plugins running while
 * another runtime owns the allocator).  The caller passes inputs and
 * outputs as for dgb_cable_assemble (comp_cable required; scratch unused).
 * The first call on a device looks up the array's device address (with that
 * device current) and should come before any stream capture.  All calls
 * share the one array: calls that overlap on the GPU race and must be
 * serialised by the caller (one stream, or events between them).  Nothing in
 * the array needs clearing; each call writes the bands before reading them.
 */
int dgb_cable_step_static(const dgb_cable_args* args, int32_t step, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DENDRA_GB300_H */
