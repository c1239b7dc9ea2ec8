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
  if (args->dtype == DGB_F32) return cable_run_t<float>(args, ch_max, st);
  return cable_run_t<double>(args, ch_max, st);
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
