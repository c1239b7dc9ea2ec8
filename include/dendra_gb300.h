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
 *   dgb_block3_solve          thomas_solve_cuda_bt, triton/bt_kernel.py:195-298
 *   dgb_block3_spd_solve      solve_bt_spd_cuda, triton/bt_spd_kernel.py:583-755
 *                             (3x3 block Thomas of the multi-layer extracellular
 *                             integrator, implicit.py:669-1136)
 *   dgb_cable_run             one Population.run over an unbranched HH cable
 *                             population: models/core.py:4555-4628 driving
 *                             integrators/core.py:769-834 and
 *                             integrators/implicit.py:569-664
 *   dgb_dhs_solve             dhs_solve_cuda, triton/dhs_kernel.py:634-651
 *   dgb_dhs_solve_forest      dhs_solve_multi_cuda, triton/dhs_kernel_multi.py:831-888
 *   dgb_dhs_block3_solve      dhs_bt_solve_cuda, triton/dhs_kernel_bt.py:465-479
 *   dgb_tree_contract_solve   tree_contraction.solve, triton/tree_contraction.py:748-768
 *                             (plan: dendra_solvers.TreeContractionPlan,
 *                             integrators/tree.py:841-867)
 *   dgb_detect_spikes         threshold_transition, networks/spiking.py:43-73
 *   dgb_pack_source_spikes    pack_source_spikes, networks/netcon_bitpack_kernel.cpp:145-149
 *   dgb_build_delivery        build_delivery, networks/netcon_bitpack_kernel.cpp:145-149
 *   dgb_build_delivery_uniform build_delivery_uniform, networks/netcon_bitpack_ops.py:669
 *   dgb_ring_enqueue          dense_fixed_delay_transition enqueue,
 *                             networks/_event_delivery.py:61-199
 *   dgb_net_window            Network.run step loop, networks/net.py:214-240 with
 *                             NetCon.advance (netcon.py:5183-5205) and
 *                             _dhs._step (integrators/tree.py:1202-1357)
 *   dgb_net_enqueue           NetCon enqueue, networks/_event_delivery.py:61-105
 *   dgb_cable_run_taped /     reverse mode of the same update: the gradient the
 *   dgb_cable_adjoint         reference takes by torch autograd through
 *                             integrators/implicit.py:569-664 (transpose solve of
 *                             ThomasSolve.backward, t_kernel_thomas.py:147-189)
 *   dgb_cable_assemble        the eager per-step assembly of the same update
 *                             (mechanism advance + membrane frame + RHS),
 *                             integrators/core.py:769-834, implicit.py:569-646
 *   dgb_two_tap_enqueue /     interpolated delays: ordered_two_tap_enqueue,
 *   dgb_two_tap_vjp /         delay_ring_two_tap_vjp, delay_ring_gather_two_tap
 *   dgb_two_tap_gather        (networks/_two_tap_enqueue_cpu.cpp:61-315) and
 *                             dense_interpolated_delay_transition
 *                             (networks/_event_delivery.py:229-308)
 *   dgb_netstim_init /        NetStim.initialize / NetStim.forward renewal,
 *   dgb_netstim_run           networks/_netstim_renewal.py:70-159
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
 * split).  Systems longer than 1024 rows run the sequential Thomas recurrence,
 * one thread per system, bit-identical to the CPU Thomas.  Replaces
 * thomas_solve_cuda_t / pcr_solve_cuda_t.
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
 * Synchronises the stream and returns DGB_ETIMEOUT if a bounded wait inside a
 * bulk-staged tridiagonal solve on this device gave up since the last call
 * (the systems of that CTA were then not solved), else DGB_OK; clears the
 * flag.  Bands, right-hand sides and solutions whose base addresses are
 * 16-byte aligned run the bulk-staged kernel (cp.async.bulk copies of each
 * tile's band slices into shared memory, completed on an mbarrier); others
 * run the register-direct kernel, with identical arithmetic.
 */
int dgb_tridiag_status(void* stream);

/* Diagnostic: polls a bulk-staged tridiagonal CTA spends on each stage wait
   before it gives up (0 = give up at the first poll; negative restores the
   default).  A wait that gave up drains its copies at the full limit. */
int dgb_tridiag_set_wait_limit(int64_t polls);

/*
 * Solve the transposed systems A^T y = g for the same bands (adjoint of
 * dgb_tridiag_solve): the transpose has sub-diagonal c and super-diagonal a.
 * Replaces the transpose solve inside ThomasSolve.backward.
 */
int dgb_tridiag_solve_transpose(int dtype, int64_t B, int64_t K,
                                const void* a, const void* b, const void* c,
                                const void* g, void* y, void* stream);

/*
 * Batched block-tridiagonal solve with 3x3 main blocks and diagonal
 * off-diagonal blocks (multi-layer extracellular cables: intracellular v and
 * two extracellular shells per compartment).  Row k of system b:
 *   diag(lower[k-1]) x[k-1] + main[k] x[k] + diag(upper[k]) x[k+1] = rhs[k]
 *   lower, upper: (B, K-1, 3); main: (B, K, 3, 3) row-major; rhs, x: (B, K, 3).
 * One warp per system: each lane eliminates its chunk of block rows (3x3
 * inverses by cofactors), the 32 reduced block rows are decoupled by block
 * PCR over warp shuffles, then back substitution; longer systems (whose
 * chunk planes exceed shared memory) run a serial block Thomas per thread.
 * work: unused (may be NULL; dgb_block3_work_size returns 0).
 * transpose = 1 solves A^T y = rhs (the adjoint solve).  x must not alias rhs.
 * Replaces thomas_solve_cuda_bt (triton/bt_kernel.py:195-262), selected by
 * _bwd_euler_bt._select_solver (integrators/implicit.py:905-950).
 */
int dgb_block3_solve(int dtype, int64_t B, int64_t K, const void* lower,
                     const void* main_blocks, const void* upper, const void* rhs,
                     void* x, void* work, int32_t transpose, void* stream);

/* Scratch bytes dgb_block3_solve needs (0: its factors stay on chip). */
size_t dgb_block3_work_size(int dtype, int64_t B, int64_t K);

/*
 * SPD block Thomas on the same systems (solve_bt_spd_cuda,
 * triton/bt_spd_kernel.py:174-370, 583-755): one thread per system; every
 * Schur block symmetrised and Cholesky-factored, with the reference's
 * diagonal shifts when it is not positive definite (info[b][k] = 1 when even
 * the last shift failed).  chol (B, K, 9) receives the factors; x must not
 * alias rhs.  dgb_block3_spd_solve_chol solves the same system again with
 * the cached factors (the backward's solve).
 */
int dgb_block3_spd_solve(int dtype, int64_t B, int64_t K, const void* lower,
                         const void* main_blocks, const void* upper, const void* rhs, void* x,
                         void* chol, int32_t* info, void* stream);
int dgb_block3_spd_solve_chol(int dtype, int64_t B, int64_t K, const void* lower,
                              const void* upper, const void* chol, const void* rhs, void* x,
                              void* stream);

/*
 * Tree solve with 3x3 blocks (multi-layer extracellular trees), B trees of K
 * nodes sharing one topology, in solver order:
 *   main (B, K, 3, 3) row-major node blocks D_i, edge (B, K, 3) the diagonal
 *   conductances g_i to the parent, rhs / x (B, K, 3);
 *   A_ii = D_i + diag(g_i) + sum_children diag(g_c),  A_ic = A_ci = -diag(g_c).
 * parent / order / layer_ptr: the reference's plan (order deepest layer
 * first); child_ptr (K+1) / child_idx (K-1): children of every node.  One
 * warp per tree, children pulled in CSR order (deterministic); 12*K*sizeof(T)
 * bytes of scratch per tree, in shared memory or, for larger trees, in a
 * stream-ordered global workspace.  transpose = 1 solves with main
 * blocks transposed (the adjoint system).  x must not alias rhs.
 * Replaces dhs_bt_solve_cuda (triton/dhs_kernel_bt.py:465-479).
 */
int dgb_dhs_block3_solve(int dtype, int64_t B, int64_t K, const void* main_blocks,
                         const void* edge, const void* rhs, const int32_t* parent,
                         const int32_t* order, const int32_t* layer_ptr, int32_t n_layers,
                         const int32_t* child_ptr, const int32_t* child_idx, void* x,
                         int32_t transpose, void* stream);

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
  /* optional second detection compartment per cable (-1: none) and its latch;
     a rising edge at either compartment counts */
  const int32_t* spk_idx2;
  int32_t* spk_below2;
  /* sizes known to the host: largest cable and total compartments */
  int32_t max_k;       /* max over cables of K */
  int32_t flags;       /* DGB_CABLE_* bits */
  int64_t n_comp;      /* cable_ptr[n_cables] */
  /* cable index of every compartment, int32[n_comp] (assembly kernel only) */
  const int32_t* comp_cable;
  /* scratch, int32[2] on the device (dgb_cable_run only): [0] work counter,
     [1] error bits after the run (0 = every cable advanced) */
  int32_t* scratch;
  /* launch tuning of the persistent kernels (dgb_cable_run, _taped, _adjoint):
     cables in flight per CTA, 1, 2 or 4, halved while the CTA's shared
     memory would exceed 227 KB.  0 = the library's choice: 4, narrowed while
     the population has fewer CTAs than the device has SMs; for dgb_cable_run
     and _taped, with lanes_mode 0 and at most one cable per SM, the
     split-gate run (DGB_CABLE_SPLIT_GATES).  The autotuner's knob. */
  int32_t warps_per_block;
  /* raster (Raster / APCount / threshold_crossing at callbacks.py:2114,
     _threshold_callbacks.py:50-53): n_rast (0..4) checked compartments per
     cable.  For cable c and check q: local compartment rast_idx[c*n_rast+q]
     (-1: none), the below latch rast_below[c*n_rast+q] (in/out, 1 = below),
     the crossing count rast_count[c*n_rast+q] (in/out, accumulates over
     calls) and the absolute step index (step0 + s + 1) of the count's k-th
     crossing in rast_steps[(c*n_rast+q)*rast_cap + k] while k < rast_cap.
     A final count above rast_cap means the later steps were not stored. */
  int32_t n_rast;
  const int32_t* rast_idx;
  int32_t* rast_below;
  int32_t* rast_count;
  int64_t* rast_steps;
  int32_t rast_cap;
  /* lanes per cable, the Thomas/PCR split of the persistent run: each lane
     eliminates ceil(K/lanes) rows (Thomas), the lanes' reduced rows are then
     solved by PCR across the lanes.  lanes_mode 0: 32 lanes for every cable.
     lanes_mode 1: the first n_lanes32 cables of `order` run 32 lanes, the next
     n_lanes16 run 16 lanes (two cables per warp), the rest 8 lanes (four per
     warp); order should list cables by non-increasing K.  A cable on 16 or 8
     lanes may have at most max(8, ceil(max_k / 32)) rows per lane (K <= 16 or
     8 times that); a longer one sets error bit 1 in scratch[1] and is skipped. */
  int32_t lanes_mode;
  int32_t n_lanes32;
  int32_t n_lanes16;
  /* full voltage recording (Recorder(("v",)), callbacks.py:522):
     trace_all[k * n_comp + g] = v of compartment g after k*rec_every steps of
     this call, k = 0 .. n_steps/rec_every, in the state dtype (NULL: off) */
  void* trace_all;
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
/* STOP_ON_SPIKE: a cable stops at the end of the step in which its first
   spike is counted (its state then holds that step; the trace is complete up
   to it).  For threshold trials, which only need to know whether a fibre fires. */
#define DGB_CABLE_STOP_ON_SPIKE 8
/* SPLIT_GATES (dgb_cable_run, dgb_cable_run_taped; lanes_mode 0): one cable
   per CTA of 4 warps, one per SM sub-partition.  The gate advance and row
   assembly of the cable's rows are spread over the 4 warps; the solve,
   detection and recording stay on the first.  The same operations as the
   one-warp run: float32 results bit for bit; float64 ones up to the last
   bits, where the compiler may contract a different multiply-add of the same
   expression.  For populations with fewer cables than SMs: one warp per cable
   leaves most of an SM's arithmetic rate unused (4 float64 cables on one SM ran
   nearly as fast as 1).  Chosen without the flag
   when warps_per_block is 0, lanes_mode is 0 and n_cables is at most the
   device's SM count. */
#define DGB_CABLE_SPLIT_GATES 16

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
 * dgb_cable_run that also writes the state tape of the run, for the adjoint:
 *   tape: (n_steps + 1, 4, n_comp) in the state dtype; tape[k][q][g] is
 *   state q (0 v, 1 m, 2 h, 3 n) of compartment g after k steps of this call.
 * n_comp must be set; DGB_CABLE_STOP_ON_SPIKE is rejected.  This is the
 * recompute pass of checkpoint-and-recompute: run it from a checkpoint over
 * one segment, then dgb_cable_adjoint over the same segment.  tape = NULL
 * runs the same kernel without writing a tape: checkpoints taken that way lie
 * on bitwise the same trajectory as the taped recompute.
 */
int dgb_cable_run_taped(const dgb_cable_args* args, void* tape, void* stream);

/*
 * Adjoint of one segment of dgb_cable_run.  The reference obtains these
 * gradients by torch autograd through the step (integrators/implicit.py:569-664,
 * mechanisms/_cnexp.py:96-132, mod/HH.py:24-40,109-116) and the transpose
 * solve of ThomasSolve.backward (triton/t_kernel_thomas.py:147-189).
 */
typedef struct dgb_cable_adjoint_args {
  const void* tape;       /* the segment's tape from dgb_cable_run_taped */
  const void* trace_grad; /* [n_cables][trace_len]: dLoss/dtrace, trace sample k
                             recorded after global step k*rec_every; NULL: none */
  int64_t trace_len;
  /* adjoint state per compartment: in, the adjoint of the state after the
     segment; out, the adjoint of the state before it */
  void* lam_v;
  void* lam_m;
  void* lam_h;
  void* lam_n;
  /* accumulated (+=) per compartment: dLoss/dgnabar, dLoss/dgkbar, dLoss/dgl */
  void* grad_gnabar;
  void* grad_gkbar;
  void* grad_gl;
  /* accumulated (+=) per compartment: lam_g * g for both axial bands
     (g_right, g_left) of the compartment's row, i.e. dLoss/dkappa_i for
     g -> kappa_i g.  The bands scale as 1/Ra, so for one Ra per cable
     dLoss/dRa = -(sum over the cable's compartments of grad_axial) / Ra.
     Every accumulator is carried through the segment in the same order as one
     uninterrupted reverse sweep, so results do not depend on the segment
     length. */
  void* grad_axial;
} dgb_cable_adjoint_args;

/*
 * Walk one segment backwards: args describes the forward segment (same
 * population, stimulus, rec_idx, rec_every, step0 and n_steps as the taped run;
 * v/m/h/n are not read).  One warp per cable; the transposed tridiagonal
 * system is solved with the same chunked elimination as the forward.
 * DGB_CABLE_FAST_MATH (float32) evaluates the gate partials with shared
 * exponentials, fast exponentials and approximate reciprocals, and the solve
 * with approximate reciprocals.  The cable size limit is set by shared memory
 * (float32: K <= 1024; float64: K <= 896 with every optional plane present).
 */
int dgb_cable_adjoint(const dgb_cable_args* args, const dgb_cable_adjoint_args* adj,
                      void* stream);

/* Diagnostic: polls a dgb_cable_adjoint warp spends on the first wait for a
   tape stage before it gives up (0 = give up at the first poll; negative
   restores the default 2^22).  A warp that gave up drains its posted copies
   at the full limit, sets error bit 4 in scratch[1] and ends.  Lets a test
   exercise the timeout path without a fault; no reference counterpart. */
int dgb_cable_adjoint_set_wait_limit(int64_t polls);

/* sizeof(dgb_cable_adjoint_args) as compiled (for foreign-language mirrors). */
size_t dgb_cable_adjoint_args_size(void);

/*
 * Tree (DHS/Hines) solve of B trees sharing one topology of K nodes, in the
 * solver order of the reference's plan (build_dhs_layers):
 *   d: (B, K) membrane diagonal, a: (B, K) axial conductance of each node to
 *   its parent (a[:, root] acts as extra diagonal), b: (B, K) right-hand
 *   side, x: (B, K) solution.  parent: (K) int32, -1 at the root; order: (K)
 *   nodes deepest layer first; layer_ptr: (n_layers + 1) layer boundaries in
 *   order; child_ptr (K + 1) / child_idx (K - 1): children of each node (CSR).
 * One warp per tree; deterministic (children summed in child_idx order, no
 * floating-point atomics).  Replaces dhs_solve_cuda
 * (dendra/models/integrators/triton/dhs_kernel.py:634-651).
 */
int dgb_dhs_solve(int dtype, int64_t B, int64_t K, const void* d, const void* a,
                  const void* b, const int32_t* parent, const int32_t* order,
                  const int32_t* layer_ptr, int32_t n_layers,
                  const int32_t* child_ptr, const int32_t* child_idx, void* x,
                  void* stream);

/* Trees of different topologies solved in one launch (packed forest). */
typedef struct dgb_forest {
  int32_t n_trees;
  int32_t max_k;                /* largest tree, in nodes */
  const int64_t* node_ptr;      /* [n_trees+1] tree t's d/a/b/x entries */
  const int32_t* plan_of;       /* [n_trees] topology plan of tree t; NULL: plan t */
  const int64_t* plan_node_ptr; /* [n_plans+1] plan p's K_p entries of parent, order
                                   and child_idx (K_p - 1 children, one unused)
                                   start at plan_node_ptr[p]; its child_ptr
                                   (K_p + 1 entries) starts at plan_node_ptr[p] + p */
  const int64_t* plan_layer_off;/* [n_plans+1] plan p's layer_ptr entries (L_p+1) */
  const int32_t* parent;        /* local node indices, per plan */
  const int32_t* order;
  const int32_t* layer_ptr;
  const int32_t* child_ptr;
  const int32_t* child_idx;
  /* optional chain schedule (NULL chain_nodes: the layer schedule above).
     Plan p's chain_nodes (K_p entries) start at plan_node_ptr[p]: unbranched
     chains one after another, each from its bottom node to its top; its
     chain_ptr (n_chains_p + 1 offsets into that block) at plan_chain_off[p];
     its chain_level (n_levels_p + 1 offsets into its chains; level-0 chains
     end in leaves, a level-l chain ends in a branch node whose child chains
     have lower levels) at plan_clevel_off[p].  Same results as the layer
     schedule; used by dgb_net_window and, one warp per tree, by
     dgb_dhs_solve_forest. */
  const int64_t* plan_chain_off;
  const int64_t* plan_clevel_off;
  const int32_t* chain_nodes;
  const int32_t* chain_ptr;
  const int32_t* chain_level;
  /* optional [n_trees] node counts for row-padded planes (dgb_dhs_solve_forest
     only): tree t's K_t nodes start at node_ptr[t], the rest of its row is
     not touched; NULL: K_t = node_ptr[t+1] - node_ptr[t] */
  const int32_t* tree_k;
} dgb_forest;

/*
 * Heterogeneous trees (different sizes and topologies) in one launch, values
 * packed by node_ptr (or in row-padded planes with tree_k).  Replaces dhs_solve_multi_cuda
 * (dendra/models/integrators/triton/dhs_kernel_multi.py:831-888).
 */
int dgb_dhs_solve_forest(int dtype, const dgb_forest* forest, const void* d,
                         const void* a, const void* b, void* x, void* stream);

/* One window of a network of branched HH-soma cells (see dgb_net_window). */
typedef struct dgb_net_args {
  int32_t dtype;
  int32_t n_cells;
  int32_t n_steps;      /* window length W <= 64, at most the minimum delay */
  int32_t bg_syn;       /* local synapse index receiving background events */
  int64_t step0;        /* global index of the window's first step */
  int64_t depth;        /* delay-ring depth (rows) */
  int64_t slot0;        /* ring row due at step0 */
  int64_t n_syn;        /* total synapses = ring width */
  dgb_forest forest;    /* the cells' trees (node-packed), plan arrays on the device */
  /* per compartment (node-packed): v in/out, area (cm^2), cm/dt (S), axial
     conductance to the parent (S, 0 at the root), leak/passive g (S/cm^2) and
     reversal (mV) */
  void* v;
  const void* area;
  const void* cm_dt;
  const void* a_geom;
  const void* gl;
  const void* el;
  /* soma (node 0 of each cell) HH gates, per cell, in/out */
  void* m;
  void* h;
  void* n;
  double gnabar, gkbar, ena, ek, q10, dt_ms, spk_thr;
  /* Exp2Syn synapses: cell c owns [syn_ptr[c], syn_ptr[c+1]); node_syn_ptr has
     K_c + 1 entries per cell (at node_ptr[c] + c) giving each node's local
     synapse range (synapses sorted by node) */
  const int64_t* syn_ptr;
  const int32_t* node_syn_ptr;
  void* syn_A;
  void* syn_B;
  const void* syn_factor;
  const void* syn_decay_A;  /* exp(-dt / tau1_effective) */
  const void* syn_decay_B;  /* exp(-dt / tau2) */
  double e_syn;
  void* ring;               /* [depth][n_syn], rows cleared as they are delivered */
  /* background events: bit (step, cell) of [steps][bg_words] uint64 words */
  const uint64_t* bg_bits;
  int64_t bg_words;
  double bg_weight;
  /* spikes: latch in/out, window spike mask out (bit s = step step0+s), count in/out */
  uint8_t* below;
  uint64_t* spike_bits;
  int32_t* spike_count;
  /* warps per CTA of dgb_net_window: 1, 2, 4 or 8 (0 = 4; at most
     max(threads_per_cell, 128) threads), reduced while the
     CTA's cells would need more than 227 KB of shared memory */
  int32_t warps_per_block;
  /* threads advancing one cell: 32, 64, 128, 256 or 512 (0 = 128); identical results.
     Both are the autotuner's knobs. */
  int32_t threads_per_cell;
  /* optional drive of the tree step (integrators/tree.py:1262-1302), NULL = none:
     extracellular ve = ve_field[node] * amp on [delay, delay + pw) of the
     cell (its edge currents g (ve_child - ve_parent) enter the parent and
     leave the child), and an injected current (mA) of a rectangular pulse at
     local node in_node[cell] (-1: none).  Pulse times are t0_ms + step dt in
     binary64, cast to the state dtype. */
  const void* ve_field;
  const void* ve_amp;
  const void* ve_delay;
  const void* ve_pw;
  const int32_t* in_node;
  const void* in_amp;
  const void* in_delay;
  const void* in_pw;
  double t0_ms;
  /* optional subset of cells advanced by this launch (NULL: every cell):
     cell_list[0 .. n_list) are cell indices; list_max_k must bound their
     sizes (it sizes the shared memory per cell in place of forest.max_k).
     Launching size classes separately (small cells with a small list_max_k,
     more of them per SM) gives the same results as one launch.  A listed
     cell larger than list_max_k is not advanced; its spike_count is set to
     INT32_MIN. */
  const int32_t* cell_list;
  int32_t n_list;
  int32_t list_max_k;
} dgb_net_args;

/* sizeof(dgb_net_args) as compiled (for foreign-language mirrors). */
size_t dgb_net_args_size(void);

/*
 * Advance every cell by n_steps steps in one launch: deliver due events into
 * Exp2Syn states, detect soma spikes, advance synapses and soma gates,
 * assemble and solve each cell's tree system (deterministic DHS), update v.
 * Replaces the per-step Network.run loop (networks/net.py:214-240) over
 * NetCon.advance (netcon.py:5183-5205) and _dhs._step (integrators/tree.py:1202-1357).
 */
int dgb_net_window(const dgb_net_args* args, void* stream);

/*
 * Enqueue a window's spikes: for every target synapse p (CSR post_ptr over
 * connections sorted by target; ring column post_col[p] or p) and each of its
 * connections e: for each window step s whose bit is set in
 * spike_bits[pre[e]], ring[(slot0 + s + delay_steps[e]) % depth][col] += weight[e].
 */
int dgb_net_enqueue(int dtype, void* ring, int64_t depth, int64_t n_syn, int64_t slot0,
                    const int64_t* post_ptr, int64_t n_post, const int64_t* post_col,
                    const int64_t* pre, const int64_t* delay_steps, const void* weight,
                    const uint64_t* spike_bits, void* stream);

/*
 * Rising-edge spike detection (threshold_transition): for each source s,
 * spikes[s] = v[comp[s]] >= thr and below[s]; then below[s] = !(v >= thr).
 * comp may be NULL (v indexed by s).  below/spikes are uint8 (0/1).
 */
int dgb_detect_spikes(int dtype, const void* v, const int64_t* comp, int64_t n,
                      double thr, uint8_t* below, uint8_t* spikes, void* stream);

/*
 * Pack a uint8 source-spike vector into row current_time_step[0] of a bit
 * history of [depth][n_words] int64 words, 63 sources per word (bit 63 unused).
 * One warp per word (ballots), no atomics.
 */
int dgb_pack_source_spikes(const uint8_t* source_spikes, int64_t n_source,
                           int64_t* packed_history, int64_t n_words,
                           const int64_t* current_time_step, void* stream);

/*
 * Delayed delivery from the bit history: for every connection e whose source
 * bit is set in row (step - delay_steps[e]) mod max_delay_steps, add
 * weight[e] to delivery_out[p] of its target p.  Connections are given in CSR
 * order by target (post_ptr, n_post + 1 entries); each target's events are
 * added one after another in connection order by one thread: deterministic,
 * no floating-point atomics.
 */
int dgb_build_delivery(int dtype, const int64_t* packed_history,
                       const int64_t* current_time_step, const int64_t* delay_steps,
                       const int64_t* conn_word_idx, const int64_t* conn_bit_mask,
                       const int64_t* post_ptr, int64_t n_post, const void* weight,
                       void* delivery_out, int64_t n_conn, int64_t max_delay_steps,
                       int64_t n_words, void* stream);

/*
 * dgb_build_delivery with one delay for every connection (delay_step, in
 * [0, max_delay_steps)): the uniform-delay launch of the reference,
 * build_delivery_uniform, networks/netcon_bitpack_ops.py:669-712 and
 * networks/netcon_bitpack_kernel.cu:95-126.  Same CSR layout and the same
 * deterministic per-target order of additions.
 */
int dgb_build_delivery_uniform(int dtype, const int64_t* packed_history,
                               const int64_t* current_time_step, int64_t delay_step,
                               const int64_t* conn_word_idx, const int64_t* conn_bit_mask,
                               const int64_t* post_ptr, int64_t n_post, const void* weight,
                               void* delivery_out, int64_t n_conn, int64_t max_delay_steps,
                               int64_t n_words, void* stream);

/*
 * Dense delay-ring enqueue: ring is [depth][width]; for each target p (CSR
 * post_ptr over connections sorted by target, column post_col[p] or p) and
 * each of its connections e with gate[pre[e]] set:
 *   ring[(slot[0] + delay_steps[e]) % depth][col] += weight[e]
 * in connection order, one thread per target.
 */
int dgb_ring_enqueue(int dtype, void* ring, int64_t depth, int64_t width,
                     const int64_t* slot, const int64_t* post_ptr, int64_t n_post,
                     const int64_t* post_col, const int64_t* pre, const uint8_t* gate,
                     const int64_t* delay_steps, const void* weight, void* stream);

/* ---------------------------------------------------------------------------
 * Threshold-proposal MLP (BF16 tensor cores, FP32 accumulation).  No
 * counterpart in the reference (it has no learned component).
 * ------------------------------------------------------------------------- */
#define DGB_EPI_PLAIN 0     /* out32 = A B */
#define DGB_EPI_BIAS 1      /* out32 = A B + bias */
#define DGB_EPI_BIAS_GELU 2 /* out32 = z = A B + bias; out16 = bf16(gelu(z)) */
#define DGB_EPI_GELU_GRAD 3 /* out16 (and out32 if given) = (A B) * gelu'(aux) */

/*
 * C[M,N] = A[M,K] B[K,N] with bf16 operands addressed by element strides
 * (A[m,k] at A + m*sam + k*sak, B[k,n] at B + k*sbk + n*sbn), fp32
 * accumulation and the epilogue above; outputs are row-major [M][N] (out16
 * bf16, out32 / bias / aux fp32).  K-major operands (sak == sbk == 1, row
 * strides multiples of 8, 16-byte aligned) with M % 128 == 0, N % 256 == 0,
 * K % 64 == 0 and K <= 256 run on tcgen05 tensor cores fed by TMA
 * (dgb_mlp_gemm_path returns 1); other shapes on mma.sync m16n8k16.
 */
int dgb_mlp_gemm(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, int64_t sak,
                 const void* B, int64_t sbk, int64_t sbn, const float* bias, int32_t epi,
                 const float* aux, float* out32, void* out16, void* stream);

/* 1 if dgb_mlp_gemm runs these arguments on the tcgen05 kernel, else 0. */
int dgb_mlp_gemm_path(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, int64_t sak,
                      const void* B, int64_t sbk, int64_t sbn);

/* Synchronises the stream and returns DGB_ETIMEOUT if a bounded wait inside
   the last tcgen05 GEMM on this device gave up (its output is then invalid).
   A load wait that gave up is recoverable: the CTA drained its copies and
   MMAs and freed its tensor memory.  If the drain gave up as well, the
   message says so and the CUDA context should be treated as unusable. */
int dgb_mlp_gemm_status(void* stream);

/* Diagnostic: polls each tcgen05 GEMM CTA spends on a TMA load wait before it
   gives up (0 = give up at the first poll; negative restores the default
   2^22).  The drain waits after a give-up always use the default.  Lets a
   test exercise the timeout path without a fault; no reference counterpart. */
int dgb_mlp_gemm_set_wait_limit(int64_t polls);

/* out[n] = sum over m of x[m][n] (fp32, fixed order). */
int dgb_colsum(int32_t M, int32_t N, const float* x, float* out, void* stream);

/* Adam step (bias-corrected, step >= 1) on fp32 weights w[n]; refreshes the
   bf16 copies w16 ([K][N], same layout) and wt16 ([N][K]) when non-null. */
int dgb_adam(int64_t n, int32_t N, int32_t K, float* w, const float* grad, float* m1, float* m2,
             float lr, float b1, float b2, float eps, int32_t step, void* w16, void* wt16,
             void* stream);

/* dy = scale * (y - target) (fp32 and/or bf16 outputs). */
int dgb_mse_grad(int64_t n, const float* y, const float* target, float scale, float* dy32,
                 void* dy16, void* stream);

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
 * device current) and should come before any stream capture; the lookup is
 * repeated if the device's context changed since (after cudaDeviceReset).  All calls
 * share the one array: calls that overlap on the GPU race and must be
 * serialised by the caller (one stream, or events between them).  Nothing in
 * the array needs clearing; each call writes the bands before reading them.
 */
int dgb_cable_step_static(const dgb_cable_args* args, int32_t step, void* stream);

/* ---------------------------------------------------------------------------
 * Interpolated (differentiable) delay transport on a dense delivery ring
 * queue[depth][width] (networks/_event_delivery.py:202-308 and the ordered
 * CPU op of networks/_two_tap_enqueue_cpu.cpp).
 *
 * Edges: weights[e], fraction[e] (upper-tap share), gates[pre_idx[e]] when
 * pre_idx is non-null (n_sources gates) else gates[e]; lower[e] / upper[e] are
 * flat ring addresses relative to the start of row *slot, in [0, depth*width):
 * the destination is (slot*width + address) mod (depth*width), its column
 * address mod width.
 *
 * Column plans: lower_ptr (width+1) / lower_edge (n_edges) list, for every
 * column, the edges whose lower address lies in it, in ascending edge order
 * (upper_ptr / upper_edge the same for upper addresses).  One thread owns one
 * column and adds its values one after another in the order of the
 * reference's CPU op, so every ring value is bit-identical to it (no
 * floating-point atomics).  A plan is a function of the addresses only; the
 * package builds it once per rollout.
 *
 * Indices are checked on the device: a slot outside [0, depth), an address
 * outside the ring, a source index outside [0, n_sources) or a plan entry that
 * does not match its column is skipped and recorded; dgb_delay_status
 * returns (and clears) the first such error.
 * ------------------------------------------------------------------------- */
#define DGB_DELAY_ERR_SLOT 1
#define DGB_DELAY_ERR_ADDRESS 2
#define DGB_DELAY_ERR_SOURCE 3
#define DGB_DELAY_ERR_PLAN 4

/*
 * ordered_two_tap_enqueue (networks/_two_tap_enqueue_cpu.cpp:61-126, in place
 * as ordered_two_tap_enqueue_ :317-328; pure-torch form
 * dense_interpolated_delay_transition, _event_delivery.py:229-308 with
 * taps = 2).  When payload is non-null it first receives row *slot (the row
 * delivered this step, dense_due); then the row is cleared and, for every
 * edge in order, queue[lower] += (w g) (1 - f), then for every edge in order
 * queue[upper] += (w g) f, each product and sum rounded separately.
 */
int dgb_two_tap_enqueue(int dtype, void* queue, int64_t depth, int64_t width,
                        const int64_t* slot, int64_t n_edges, const void* weights,
                        const void* gates, const int64_t* pre_idx, int64_t n_sources,
                        const void* fraction, const int64_t* lower, const int64_t* upper,
                        const int64_t* lower_ptr, const int64_t* lower_edge,
                        const int64_t* upper_ptr, const int64_t* upper_edge, void* payload,
                        void* stream);

/*
 * Three-tap form of the same transition (_event_delivery.py:294-306): for
 * every edge in order and tap t = 0, 1, 2,
 *   queue[((slot + offsets[e][t]) mod depth) * width + post_idx[e]] += (w g) coeff[e][t].
 * post_ptr / post_edge: edges by post column in ascending order.
 */
int dgb_three_tap_enqueue(int dtype, void* queue, int64_t depth, int64_t width,
                          const int64_t* slot, int64_t n_edges, const void* weights,
                          const void* gates, const int64_t* pre_idx, int64_t n_sources,
                          const void* coeff, const int64_t* offsets, const int64_t* post_idx,
                          const int64_t* post_ptr, const int64_t* post_edge, void* payload,
                          void* stream);

/*
 * delay_ring_gather_two_tap (_two_tap_enqueue_cpu.cpp:206-233):
 * lower_values[e] = ring[wrap(lower[e] + offset)], upper_values likewise,
 * wrap = remainder modulo ring_size.  offset is a device scalar.
 */
int dgb_two_tap_gather(int dtype, const void* ring, int64_t ring_size, const int64_t* offset,
                       int64_t n_edges, const int64_t* lower, const int64_t* upper,
                       void* lower_values, void* upper_values, void* stream);

/*
 * delay_ring_two_tap_vjp (_two_tap_enqueue_cpu.cpp:235-315) and the unfused
 * adjoint of _two_tap_enqueue.py:94-150: with lo / hi the cotangent ring read
 * at the two taps,
 *   dw = (hi f + lo (1 - f)) g,  dg = (hi f + lo (1 - f)) w,
 *   df = hi (w g) - lo (w g).
 * With pre_idx, grad_gates[s] sums its edges' dg in ascending edge order from
 * +0 (index_select_backward); source_ptr (n_sources+1) / source_edge list the
 * edges of every source in ascending order.  grad_queue is the cotangent with
 * row slot cleared; the caller forms it.
 */
int dgb_two_tap_vjp(int dtype, const void* ring, int64_t ring_size, const int64_t* offset,
                    int64_t n_edges, const void* weights, const void* gates,
                    const int64_t* pre_idx, int64_t n_sources, const void* fraction,
                    const int64_t* lower, const int64_t* upper, const int64_t* source_ptr,
                    const int64_t* source_edge, void* grad_weights, void* grad_gates,
                    void* grad_fraction, void* stream);

/*
 * Cotangents of the three-tap enqueue, gates per edge (the derivative torch
 * autograd takes through _event_delivery.py:294-306): with gv_t the ring
 * cotangent at tap t, grad_coeff[e][t] = gv_t (w g) and, with
 * s = (gv_0 c_0 + gv_1 c_1) + gv_2 c_2, grad_weights = s g, grad_gates = s w.
 */
int dgb_three_tap_vjp(int dtype, const void* ring, int64_t depth, int64_t width,
                      const int64_t* slot, int64_t n_edges, const void* weights,
                      const void* gates, const void* coeff, const int64_t* offsets,
                      const int64_t* post_idx, void* grad_weights, void* grad_gates,
                      void* grad_coeff, void* stream);

/*
 * Multi-step rollout of dgb_two_tap_enqueue in one launch, in place on ring:
 * n_steps consecutive steps from row *slot (advancing by one, modulo depth,
 * every step); gates[k] holds step k's gates (row stride n_sources, or n_edges
 * without pre_idx) and payload[k] (optional) step k's delivered row.  Both
 * taps of every edge must lie in one column: col_ptr (width+1) / col_edge list
 * each column's edges ascending, and lower_row[j] / upper_row[j], in
 * [0, depth), are the row distances of the two taps of the edge at list
 * position j (its flat addresses divided by width).  One thread owns one
 * column for the whole rollout, its ring depth held in shared memory when it
 * fits; each value is bit-identical to n_steps dgb_two_tap_enqueue calls.
 * flags: DGB_ROLLOUT_ONE_EDGE (no column holds more than one edge: a leaner
 * kernel; a column with more is skipped and reported), DGB_ROLLOUT_EMPTY_START
 * (ring contents ignored, the rollout starts from zeros),
 * DGB_ROLLOUT_NO_FINAL (the ring is not written back at the end),
 * DGB_ROLLOUT_CHAINED (every column has at most one edge, with taps at lo and
 * lo + 1, 1 <= lo <= depth - 2: the cell delivered at step k then holds
 * (c0 + upper tap of step k-lo-1) + lower tap of step k-lo, so every step is
 * computed independently, with no ring held during the rollout; a column that
 * breaks the promise is skipped and reported), DGB_ROLLOUT_GATES_BY_SOURCE
 * (with pre_idx and CHAINED: gates given per source, gates[s][k], rows of
 * gate_row >= n_steps values; see dgb_gates_by_source).
 * depth*width, n_edges and n_sources below 2^31.
 */
#define DGB_ROLLOUT_ONE_EDGE 1
#define DGB_ROLLOUT_EMPTY_START 2
#define DGB_ROLLOUT_NO_FINAL 4
#define DGB_ROLLOUT_CHAINED 8
#define DGB_ROLLOUT_GATES_BY_SOURCE 16
int dgb_two_tap_rollout(int dtype, void* ring, int64_t depth, int64_t width,
                        const int64_t* slot, int64_t n_steps, int64_t n_edges,
                        const void* weights, const void* gates, int64_t gate_row,
                        const int64_t* pre_idx,
                        int64_t n_sources, const void* fraction, const int64_t* col_ptr,
                        const int64_t* col_edge, const int32_t* lower_row,
                        const int32_t* upper_row, int32_t flags, void* payload, void* stream);

/*
 * Reverse sweep of dgb_two_tap_rollout over the same n_steps (newest first),
 * in place on the cotangent ring grad_ring (in: after the rollout, ignored
 * with DGB_ROLLOUT_EMPTY_START; out: before it).  grad_payload[k] (optional)
 * is the cotangent of step k's delivered row; it replaces the cotangent of row
 * slot_k, which the forward cleared.  Per step the VJP of dgb_two_tap_vjp;
 * grad_weights / grad_fraction accumulate over steps newest first (stored, not
 * added, at the newest step when accumulate == 0).  grad_gates[k] receives
 * step k's gate cotangents; with pre_idx the per-edge values go to
 * edge_scratch[j][k] (j = list position; rows of kc = n_steps rounded up to 8
 * values, n_edges * kc in all, 32-byte aligned) and are summed per source in
 * ascending edge order: source_ptr (n_sources+1) / source_pos give each
 * source's edges, ascending by edge, as list positions.
 */
int dgb_two_tap_rollout_vjp(int dtype, void* grad_ring, int64_t depth, int64_t width,
                            const int64_t* slot, int64_t n_steps, int64_t n_edges,
                            const void* weights, const void* gates, int64_t gate_row,
                            const int64_t* pre_idx,
                            int64_t n_sources, const void* fraction, const int64_t* col_ptr,
                            const int64_t* col_edge, const int32_t* lower_row,
                            const int32_t* upper_row, int32_t flags, const int64_t* source_ptr,
                            const int64_t* source_pos, const void* grad_payload,
                            int32_t accumulate, void* grad_weights, void* grad_gates,
                            void* grad_fraction, void* edge_scratch, void* stream);

/* gates_t[s][k] = gates[k][s] for k < n_steps (rows of gate_row >= n_steps
   values): the per-source layout of DGB_ROLLOUT_GATES_BY_SOURCE. */
int dgb_gates_by_source(int dtype, int64_t n_steps, int64_t n_sources, const void* gates,
                        void* gates_t, int64_t gate_row, void* stream);

/* ---------------------------------------------------------------------------
 * NetStim renewal generators (networks/_netstim_renewal.py:70-159), one
 * thread per generator.  Draws: Philox4x32-10 with key seed and counter
 * (step, generator), E = -ln(U) evaluated with rounded IEEE operations only
 * (reproducible on any host), or a caller-supplied table `draws`.
 * ------------------------------------------------------------------------- */

/* Initial clocks (netstim_initial_state): next_time = start + (noise interval) E
   when any_noise (any generator has noise > 0), else start; counts = 0.
   draws (optional): n initial draws. */
int dgb_netstim_init(int dtype, int64_t n, const void* interval, const void* noise,
                     const void* start, int32_t any_noise, uint64_t seed, const void* draws,
                     void* next_time, int64_t* counts, void* stream);

/* n_steps renewal steps (netstim_renewal without calendars) from absolute
   step step0, t = t0 + step*dt in the state dtype: a generator fires when
   t >= next_time and counts < number (NULL: unlimited); on firing next_time
   advances by interval (1 - noise) + (interval noise) E and counts by one; a
   draw is consumed every step.  draws (optional): [n_steps][n].  Outputs
   (optional): spikes[k][g] (uint8) and bits[k][n_words] (bit g & 63 of word
   g >> 6, as dgb_net_args.bg_bits). */
int dgb_netstim_run(int dtype, int64_t n, int64_t n_steps, int64_t step0, double t0, double dt,
                    const void* interval, const void* noise, const int64_t* number,
                    uint64_t seed, const void* draws, void* next_time, int64_t* counts,
                    uint8_t* spikes, uint64_t* bits, int64_t n_words, void* stream);

/* ---------------------------------------------------------------------------
 * Tree contraction (conductance form).  Plan tables are int32 device arrays
 * as built by
 * dendra_gb300/contraction.py (build_contraction_tables):
 *   seg        [n_segments][8]   ancestor, child (retained indices), interior start,
 *                                end, first interior node, stride (+1/-1 when the
 *                                run's node ids are consecutive, else 0), child
 *                                node, ancestor node
 *   interior   [n_interior]      node ids, each segment top to bottom
 *   retained   [n_retained][8]   node, incoming segment (-1), endpoint start, count,
 *                                the first four endpoints as 2*segment + side (-1)
 *   endpoint   [n_endpoints][2]  segment, side (0 ancestor end, 1 child end)
 *   round_ptr  [2][n_rounds+1]   update offsets, recovery offsets
 *   update     [n_updates][4]    source state slot, incidence start, count, 0
 *   incidence  [n_incidence][4]  removed state slot, near edge, far edge (-1),
 *                                bridge slot written (-1)
 *   recovery   [n_eliminated][8] retained index, state slot, ancestor, child (-1),
 *                                near edge, far edge (-1), 0, 0
 *   roots      [2][n_roots]      retained index, final state slot
 * seg, retained, update, incidence and recovery are 16-byte records (vector
 * loads) and must start on 16-byte boundaries; endpoint on 8 bytes.  Every slot index must lie inside its table
 * (the builder checks this).
 * ------------------------------------------------------------------------- */
typedef struct dgb_contract_plan {
  int32_t size, n_segments, n_interior, n_retained;
  int32_t n_endpoints, n_rounds, n_updates, n_incidence;
  int32_t n_eliminated, n_roots, n_bridges;
  int32_t threads; /* threads per batch row: 32, 64, 128 or 256; 0 picks by the plan's width */
  const int32_t* seg;
  const int32_t* interior;
  const int32_t* retained;
  const int32_t* endpoint;
  const int32_t* round_ptr;
  const int32_t* update;
  const int32_t* incidence;
  const int32_t* recovery;
  const int32_t* roots;
} dgb_contract_plan;

/* B scalar Hines systems of plan->size nodes sharing the plan's topology:
 * d (shunt), g (conductance to the parent; a root's g is a second shunt), rhs
 * and x are (B, K) row-major:  d_i x_i + g_i (x_i - x_p(i)) + sum_c g_c (x_i - x_c)
 * = rhs_i.  One block per row, scratch in shared memory, or in the caller's
 * workspace when it does not fit; correctly rounded operations only.  x
 * must not alias an input.  Replaces tree_contraction.solve
 * (triton/tree_contraction.py:748-768; kernels :14-480). */
int dgb_tree_contract_solve(int dtype, int64_t B, const dgb_contract_plan* plan, const void* d,
                            const void* g, const void* rhs, void* x, void* work,
                            size_t work_bytes, void* stream);

/* Workspace bytes dgb_tree_contract_solve needs for B rows: 0 when a row's
 * scratch fits in shared memory, else (rows in flight) x (the row's scratch)
 * for the same program run from global memory (trees of any size). */
size_t dgb_tree_contract_work_size(int dtype, const dgb_contract_plan* plan, int64_t B);

/* sizeof(dgb_contract_plan), for bindings that mirror the struct. */
size_t dgb_contract_plan_size(void);

/* First device-side index error of the delay kernels since the last call
   (0 = none, else DGB_DELAY_ERR_*), cleared on read; synchronises stream. */
int dgb_delay_status(void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DENDRA_GB300_H */
