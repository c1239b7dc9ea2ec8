// C-ABI entry points of the unbranched HH cable kernels; the kernels live in
// cable_impl.cuh and are compiled per dtype in cable_f32.cu / cable_f64.cu only.
#include "cable_decl.cuh"

using namespace dgb;

extern "C" int dgb_cable_run(const dgb_cable_args* args, void* stream) {
  clear_error();
  int rc = validate_cable_args(args);
  if (rc) return rc;
  DGB_REQUIRE(args->scratch != nullptr, "scratch (2 x int32, device) is required");
  if (args->n_cables == 0) return DGB_OK;
  // the largest cable decides the shared-memory block size
  const int64_t kmax = args->max_k;
  DGB_REQUIRE(kmax >= 1 && kmax <= 32 * kCableMaxCH,
              "max compartments per cable (max_k) must be in [1, %d], got %lld",
              32 * kCableMaxCH, (long long)kmax);
  // shared memory is sized for the largest chunk (rows per lane) of any cable
  const int ch_max = (int)((kmax + 31) / 32);
  cudaStream_t st = as_stream(stream);
  if (args->dtype == DGB_F64) return cable_run_launch<double, false, false>(args, nullptr, ch_max, st);
  if (args->flags & DGB_CABLE_FAST_MATH)
    return cable_run_launch<float, true, false>(args, nullptr, ch_max, st);
  return cable_run_launch<float, false, false>(args, nullptr, ch_max, st);
}

extern "C" int dgb_cable_assemble(const dgb_cable_args* args, int32_t step, void* lower,
                                  void* main_diag, void* upper, void* rhs, void* stream) {
  clear_error();
  int rc = validate_cable_args(args);
  if (rc) return rc;
  DGB_REQUIRE(args->comp_cable != nullptr,
              "comp_cable (cable index per compartment, int32[n_comp]) is required");
  DGB_REQUIRE(lower && main_diag && upper && rhs, "band outputs must be non-null");
  if (args->n_comp == 0) return DGB_OK;
  cudaStream_t st = as_stream(stream);
  if (args->dtype == DGB_F32)
    return cable_assemble_t<float>(args, step, lower, main_diag, upper, rhs, st);
  return cable_assemble_t<double>(args, step, lower, main_diag, upper, rhs, st);
}

extern "C" int dgb_cable_solve_update(const dgb_cable_args* args, const void* lower,
                                      const void* main_diag, const void* upper, const void* rhs,
                                      void* stream) {
  clear_error();
  int rc = validate_cable_args(args);
  if (rc) return rc;
  DGB_REQUIRE(lower && main_diag && upper && rhs, "band inputs must be non-null");
  if (args->n_cables == 0) return DGB_OK;
  const int64_t kmax = args->max_k;
  DGB_REQUIRE(kmax >= 1 && kmax <= 32 * kSolveUpdateMaxCH,
              "max compartments per cable (max_k) must be in [1, %d], got %lld",
              32 * kSolveUpdateMaxCH, (long long)kmax);
  cudaStream_t st = as_stream(stream);
  if (args->dtype == DGB_F32)
    return cable_solve_update_t<float>(args, lower, main_diag, upper, rhs, st);
  return cable_solve_update_t<double>(args, lower, main_diag, upper, rhs, st);
}

static int validate_taped(const dgb_cable_args* args) {
  DGB_REQUIRE(args->scratch != nullptr, "scratch (2 x int32, device) is required");
  DGB_REQUIRE(args->n_comp >= 0, "n_comp must be the total compartment count");
  DGB_REQUIRE((args->flags & DGB_CABLE_STOP_ON_SPIKE) == 0,
              "the taped run and the adjoint cover every step of the segment "
              "(DGB_CABLE_STOP_ON_SPIKE is not accepted)");
  const int64_t kmax = args->max_k;
  DGB_REQUIRE(kmax >= 1 && kmax <= 32 * kCableMaxCH,
              "max compartments per cable (max_k) must be in [1, %d], got %lld",
              32 * kCableMaxCH, (long long)kmax);
  return DGB_OK;
}

extern "C" int dgb_cable_run_taped(const dgb_cable_args* args, void* tape, void* stream) {
  clear_error();
  int rc = validate_cable_args(args);
  if (rc) return rc;
  rc = validate_taped(args);
  if (rc) return rc;
  if (args->n_cables == 0) return DGB_OK;
  const int ch_max = (args->max_k + 31) / 32;
  cudaStream_t st = as_stream(stream);
  if (args->dtype == DGB_F64) return cable_run_launch<double, false, true>(args, tape, ch_max, st);
  if (args->flags & DGB_CABLE_FAST_MATH)
    return cable_run_launch<float, true, true>(args, tape, ch_max, st);
  return cable_run_launch<float, false, true>(args, tape, ch_max, st);
}

extern "C" int dgb_cable_adjoint_set_wait_limit(int64_t polls) {
  clear_error();
  const int rc = cable_adjoint_wait_limit_t<float>(polls);
  if (rc) return rc;
  return cable_adjoint_wait_limit_t<double>(polls);
}

extern "C" int dgb_cable_adjoint(const dgb_cable_args* args, const dgb_cable_adjoint_args* adj,
                                 void* stream) {
  clear_error();
  int rc = validate_cable_args(args);
  if (rc) return rc;
  rc = validate_taped(args);
  if (rc) return rc;
  DGB_REQUIRE(adj != nullptr && adj->tape != nullptr, "adjoint args with a tape are required");
  DGB_REQUIRE(adj->lam_v && adj->lam_m && adj->lam_h && adj->lam_n,
              "lam_v, lam_m, lam_h and lam_n are required");
  DGB_REQUIRE(adj->grad_gnabar && adj->grad_gkbar && adj->grad_gl && adj->grad_axial,
              "grad_gnabar, grad_gkbar, grad_gl and grad_axial are required");
  DGB_REQUIRE(!adj->trace_grad || (args->rec_idx && adj->trace_len >= 0),
              "trace_grad requires rec_idx and trace_len >= 0");
  if (args->n_cables == 0) return DGB_OK;
  const int ch_max = (args->max_k + 31) / 32;
  cudaStream_t st = as_stream(stream);
  if (args->dtype == DGB_F32) return cable_adjoint_t<float>(args, adj, ch_max, st);
  return cable_adjoint_t<double>(args, adj, ch_max, st);
}
