// Declarations shared by the cable C-ABI translation unit and the per-dtype
// kernel translation units (cable_f32.cu, cable_f64.cu).  Kernel templates
// live in cable_impl.cuh and are compiled only by the per-dtype units, so each
// kernel has exactly one definition in the library.
#pragma once

#include "common.cuh"

namespace dgb {

constexpr int kCableMaxCH = 32;        // persistent run: K <= 1024
constexpr int kSolveUpdateMaxCH = 16;  // plain per-step solve: K <= 512

// Persistent run of one (dtype, arithmetic, tape) variant; each variant is
// compiled in its own translation unit (cable_run_*.cu, cable_taped_*.cu).
template <typename T, bool FAST, bool TAPE>
int cable_run_launch(const dgb_cable_args* args, void* tape, int ch_max, cudaStream_t st);
template <typename T>
int cable_adjoint_t(const dgb_cable_args* args, const dgb_cable_adjoint_args* adj, int ch_max,
                    cudaStream_t st);
template <typename T>
int cable_adjoint_wait_limit_t(int64_t polls);
template <typename T>
int cable_assemble_t(const dgb_cable_args* args, int32_t step, void* lower, void* mainv,
                     void* upper, void* rhs, cudaStream_t st);
template <typename T>
int cable_solve_update_t(const dgb_cable_args* args, const void* lower, const void* mainv,
                         const void* upper, const void* rhs, cudaStream_t st);

inline int validate_cable_args(const dgb_cable_args* a) {
  DGB_REQUIRE(a != nullptr, "args must be non-null");
  DGB_REQUIRE(a->dtype == DGB_F32 || a->dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(a->n_cables >= 0 && a->n_steps >= 0, "n_cables and n_steps must be >= 0");
  DGB_REQUIRE(a->cable_ptr && a->v && a->m && a->h && a->n, "cable_ptr and v/m/h/n are required");
  DGB_REQUIRE(a->g_right && a->g_left && a->scale && a->cm_inv,
              "g_right, g_left, scale and cm_inv are required");
  DGB_REQUIRE(a->gnabar && a->gkbar && a->gl && a->el, "gnabar, gkbar, gl and el are required");
  DGB_REQUIRE(!a->in_idx || (a->in_amp && a->in_delay && a->in_pw),
              "in_idx requires in_amp, in_delay and in_pw");
  DGB_REQUIRE(!a->ve_amp || (a->field && a->ve_delay && a->ve_pw),
              "ve_amp requires field, ve_delay and ve_pw");
  DGB_REQUIRE(!a->spk_idx || (a->spk_below && a->spk_count && a->spk_first),
              "spk_idx requires spk_below, spk_count and spk_first");
  DGB_REQUIRE(!a->trace || a->rec_idx, "trace requires rec_idx");
  DGB_REQUIRE(!a->spk_idx2 || (a->spk_idx && a->spk_below2),
              "spk_idx2 requires spk_idx and spk_below2");
  DGB_REQUIRE(a->rec_every >= 1, "rec_every must be >= 1");
  DGB_REQUIRE((a->flags & ~(DGB_CABLE_UNIFORM_CHANNELS | DGB_CABLE_UNIFORM_GEOMETRY |
                             DGB_CABLE_FAST_MATH | DGB_CABLE_STOP_ON_SPIKE |
                             DGB_CABLE_SPLIT_GATES)) == 0,
              "unknown flags %d", a->flags);
  DGB_REQUIRE(!(a->flags & DGB_CABLE_FAST_MATH) || a->dtype == DGB_F32,
              "DGB_CABLE_FAST_MATH applies to float32 state only");
  DGB_REQUIRE(a->warps_per_block >= 0 && a->warps_per_block <= 4 && a->warps_per_block != 3,
              "warps_per_block must be 0 (default), 1, 2 or 4, got %d", a->warps_per_block);
  DGB_REQUIRE(a->n_rast >= 0 && a->n_rast <= 4, "n_rast must be in [0, 4], got %d", a->n_rast);
  DGB_REQUIRE(a->n_rast == 0 || (a->rast_idx && a->rast_below && a->rast_count),
              "n_rast > 0 requires rast_idx, rast_below and rast_count");
  DGB_REQUIRE(a->n_rast == 0 || a->rast_cap >= 0, "rast_cap must be >= 0");
  DGB_REQUIRE(a->n_rast == 0 || a->rast_cap == 0 || a->rast_steps,
              "rast_cap > 0 requires rast_steps");
  DGB_REQUIRE(a->lanes_mode == 0 || a->lanes_mode == 1, "lanes_mode must be 0 or 1");
  DGB_REQUIRE(a->lanes_mode == 0 ||
                  (a->n_lanes32 >= 0 && a->n_lanes16 >= 0 &&
                   (int64_t)a->n_lanes32 + a->n_lanes16 <= a->n_cables),
              "n_lanes32 + n_lanes16 must lie in [0, n_cables]");
  DGB_REQUIRE(!a->trace_all || a->n_comp >= 0, "trace_all requires n_comp");
  return DGB_OK;
}

}  // namespace dgb
