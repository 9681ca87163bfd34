// frontend_check.cpp -- SANKHYA's own front ends reaching the GB300 seam, on the CPU.
//
// Linked with the reference's whole core (solve(), presolve, the engines, the readers and the
// C API, compiled as a CUDA build compiles them), the seam files that replace src/gpu
// (seam/pdhg_gpu.cpp, pdhg_multi_gpu.cpp, gpu_memory.cpp, device.cpp) and the C-ABI stand-in
// (seam_standin.cpp), which answers the device probes and runs the reference's CPU PDHG
// behind the engine's calls. argv[1] is an MPS model. Checks:
//  1. an engine that cannot be created: solve() with gpu=true returns kNumericalError with
//     the engine's message and runs no CPU PDHG in its place;
//  2. solve() with algorithm=pdhg and gpu=true reaches the seam once and returns what the CPU
//     route (gpu=false) returns, bit for bit: status, iterations, objective, the three
//     vectors; with and without the interior-point polish that follows PDHG by default;
//  3. gpu_devices="0,1" reaches the same engine through solve_pdhg_multi_gpu;
//  4. the gates of src/core/solve.cpp:733-773 run on the seam's answers: deterministic=true,
//     a compute capability below 10.3 and too little free memory each keep the solve on the
//     reference's CPU PDHG;
//  5. algorithm=auto routes a model of 100,000 rows to the GPU when the device answers;
//  6. the C API (sankhya_solve with the gpu option set) reaches the seam;
//  7. the version banner names the device the seam reports;
//  8. tests/unit/test_multi_gpu.cpp:191-228 restated: solve_pdhg_multi_gpu with the virtual
//     devices {0, 0} gives the single-device answer (afiro, 1e-6, no polish). The reference
//     expects its own "pdhg-cuda-multi" algorithm name there; this seam keeps an LP on one
//     device and says "pdhg-gpu".
//
// `frontend_check --write model.mps out.sol` instead solves the model once through solve()
// with algorithm=pdhg, gpu=true (tolerance 1e-8, no polish) and writes the answer with the
// reference's own writer (io::write_solution), for the reference's independent verifier
// (tools/verify_solution.py). It fails if the solve did not go through the seam.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sankhya/io.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/sankhya.h"
#include "sankhya/version.hpp"
#include "gpu/pdhg_gpu.hpp"
#include "gpu/pdhg_multi_gpu.hpp"

extern "C" {
void standin_fail_create(int fail);
void standin_set_device(int available, int major, int minor, unsigned long long free_bytes,
                        unsigned long long total_bytes, unsigned long long estimate);
long long standin_solve_count(void);
}

namespace {

int g_failures = 0;

void check(bool ok, const std::string& what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what.c_str());
    ++g_failures;
  }
}

bool same(const std::vector<double>& a, const std::vector<double>& b) {
  return a.size() == b.size() &&
         (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(double)) == 0);
}

bool same(double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; }

sankhya::Options pdhg_options(bool gpu, bool polish) {
  sankhya::Options o;
  o.set_bool("log_to_console", false);
  o.set_string("algorithm", "pdhg");
  o.set_bool("gpu", gpu);
  o.set_bool("pdhg_polish", polish);
  o.set_double("pdhg_tolerance", 1e-6);
  o.set_int("iteration_limit", 200000);
  return o;
}

void check_same_answer(const sankhya::Solution& gpu, const sankhya::Solution& cpu,
                       const std::string& what) {
  check(gpu.status == cpu.status, what + ": status");
  check(gpu.iterations == cpu.iterations, what + ": iterations");
  check(same(gpu.objective, cpu.objective), what + ": objective");
  check(same(gpu.col_value, cpu.col_value), what + ": col_value");
  check(same(gpu.col_dual, cpu.col_dual), what + ": col_dual");
  check(same(gpu.row_dual, cpu.row_dual), what + ": row_dual");
}

// A reached-the-seam check: the stand-in's solve count moves by exactly `expected`.
struct Route {
  long long before = standin_solve_count();
  bool moved_by(long long expected) const { return standin_solve_count() - before == expected; }
};

// 100,000 rows x_i + x_{i+1} >= 1 over 100,001 columns: large enough for the automatic
// selection's GPU rule (kPdhgRowFloor, src/core/engine_selection.hpp:53).
sankhya::Model chain_model() {
  const int m = 100000, n = m + 1;
  sankhya::Model model;
  model.col_cost.assign(n, 1.0);
  model.col_lower.assign(n, 0.0);
  model.col_upper.assign(n, sankhya::kInfinity);
  model.col_type.assign(n, sankhya::VarType::kContinuous);
  model.row_lower.assign(m, 1.0);
  model.row_upper.assign(m, sankhya::kInfinity);
  model.matrix.reset(m, n);
  for (int i = 0; i < m; ++i) {
    model.matrix.add_entry(i, i, 1.0);
    model.matrix.add_entry(i, i + 1, 1.0);
  }
  model.matrix.finalize();
  return model;
}

}  // namespace

// Solve through the seam and write the reference's .sol file.
int write_mode(const char* model_path, const char* sol_path) {
  sankhya::Model model;
  const sankhya::io::ReadResult read = sankhya::io::read_model(model_path, &model);
  if (!read.ok) {
    std::printf("cannot read %s: %s\n", model_path, read.error.c_str());
    return 2;
  }
  sankhya::Options o = pdhg_options(true, false);
  o.set_double("pdhg_tolerance", 1e-8);
  o.set_int("iteration_limit", 1000000);
  const Route route;
  const sankhya::Solution s = sankhya::solve(model, o);
  std::string error;
  if (!sankhya::io::write_solution(sol_path, model, s, o, &error)) {
    std::printf("cannot write %s: %s\n", sol_path, error.c_str());
    return 2;
  }
  std::printf("%s: %s, %lld iterations, objective %.17g, algorithm %s\n", model_path,
              sankhya::to_string(s.status), static_cast<long long>(s.iterations),
              s.objective, s.algorithm.c_str());
  return route.moved_by(1) ? 0 : 1;
}

int main(int argc, char** argv) {
  if (argc == 4 && std::strcmp(argv[1], "--write") == 0) return write_mode(argv[2], argv[3]);
  if (argc < 2) {
    std::printf("usage: frontend_check model.mps | frontend_check --write model.mps out.sol\n");
    return 2;
  }
  sankhya::Model model;
  const sankhya::io::ReadResult read = sankhya::io::read_model(argv[1], &model);
  if (!read.ok) {
    std::printf("cannot read %s: %s\n", argv[1], read.error.c_str());
    return 2;
  }

  // 1. No engine: an error status with the engine's message, no CPU PDHG instead. This runs
  //    first because the seam keeps the engine it creates for the rest of the process.
  {
    standin_fail_create(1);
    const Route route;
    const sankhya::Solution s = sankhya::solve(model, pdhg_options(true, false));
    check(s.status == sankhya::SolveStatus::kNumericalError, "no engine: kNumericalError");
    check(s.message.find("no usable CUDA device") != std::string::npos,
          "no engine: the engine's message is kept (" + s.message + ")");
    check(route.moved_by(0), "no engine: nothing solved");
    standin_fail_create(0);
  }

  // 2. The GPU route and the CPU route give the same answer.
  for (const bool polish : {false, true}) {
    const std::string what = polish ? "solve() with the polish" : "solve()";
    const sankhya::Solution cpu = sankhya::solve(model, pdhg_options(false, polish));
    const Route route;
    const sankhya::Solution gpu = sankhya::solve(model, pdhg_options(true, polish));
    check(route.moved_by(1), what + ": the seam ran once");
    check(gpu.algorithm.find("gpu") != std::string::npos,
          what + ": algorithm names the GPU (" + gpu.algorithm + ")");
    check(cpu.algorithm.find("gpu") == std::string::npos, what + ": CPU route stays on the CPU");
    check(gpu.status == sankhya::SolveStatus::kOptimal, what + ": optimal");
    check_same_answer(gpu, cpu, what);
  }

  const sankhya::Solution reference = sankhya::solve(model, pdhg_options(false, false));

  // 3. Two device ids: solve_pdhg_multi_gpu, which keeps the LP on one device.
  {
    sankhya::Options o = pdhg_options(true, false);
    o.set_string("gpu_devices", "0,1");
    const Route route;
    const sankhya::Solution s = sankhya::solve(model, o);
    check(route.moved_by(1), "gpu_devices=0,1: the seam ran once");
    check_same_answer(s, reference, "gpu_devices=0,1");
  }

  // 4. The gates run on the seam's probes and keep the solve on the CPU.
  {
    sankhya::Options o = pdhg_options(true, false);
    o.set_bool("deterministic", true);
    const Route route;
    const sankhya::Solution s = sankhya::solve(model, o);
    check(route.moved_by(0), "deterministic: not routed to the GPU");
    check_same_answer(s, reference, "deterministic");
  }
  {
    standin_set_device(1, 9, 0, 280ULL << 30, 284ULL << 30, 64ULL << 20);
    const Route route;
    const sankhya::Solution s = sankhya::solve(model, pdhg_options(true, false));
    check(route.moved_by(0), "compute capability 9.0: not routed to the GPU");
    check_same_answer(s, reference, "compute capability 9.0");
  }
  {
    // 30 GiB free against a 10 GiB estimate plus the reserve (10% of 284 GiB).
    standin_set_device(1, 10, 3, 30ULL << 30, 284ULL << 30, 10ULL << 30);
    const Route route;
    const sankhya::Solution s = sankhya::solve(model, pdhg_options(true, false));
    check(route.moved_by(0), "too little free memory: not routed to the GPU");
    check_same_answer(s, reference, "too little free memory");
    standin_set_device(1, 10, 3, 280ULL << 30, 284ULL << 30, 64ULL << 20);
    const Route fits;
    const sankhya::Solution t = sankhya::solve(model, pdhg_options(true, false));
    check(fits.moved_by(1), "enough free memory: routed to the GPU");
    check_same_answer(t, reference, "enough free memory");
  }

  // 5. algorithm=auto on 100,000 rows picks GPU PDHG when the device answers, and the CPU
  //    PDHG when it does not.
  {
    const sankhya::Model chain = chain_model();
    sankhya::Options o;
    o.set_bool("log_to_console", false);
    o.set_string("algorithm", "auto");
    o.set_bool("presolve", false);
    o.set_bool("pdhg_polish", false);
    o.set_int("iteration_limit", 80);
    const Route route;
    const sankhya::Solution s = sankhya::solve(chain, o);
    check(route.moved_by(1), "auto, 100,000 rows: routed to the GPU");
    check(s.algorithm.find("gpu") != std::string::npos,
          "auto, 100,000 rows: algorithm names the GPU (" + s.algorithm + ")");
    check(s.iterations == 80, "auto, 100,000 rows: iteration limit honoured");
    standin_set_device(0, 0, 0, 0, 0, 0);
    const Route none;
    const sankhya::Solution c = sankhya::solve(chain, o);
    check(none.moved_by(0), "auto, no device: CPU PDHG");
    check(c.algorithm.find("gpu") == std::string::npos, "auto, no device: CPU algorithm");
    standin_set_device(1, 10, 3, 280ULL << 30, 284ULL << 30, 64ULL << 20);
  }

  // 6. The C API.
  {
    sankhya_model* cm = sankhya_model_create();
    check(sankhya_model_read(cm, argv[1]) == SANKHYA_OK, "C API: model read");
    sankhya_options* co = sankhya_options_create();
    sankhya_options_set_bool(co, "log_to_console", 0);
    sankhya_options_set_string(co, "algorithm", "pdhg");
    sankhya_options_set_bool(co, "gpu", 1);
    sankhya_options_set_bool(co, "pdhg_polish", 0);
    sankhya_options_set_double(co, "pdhg_tolerance", 1e-6);
    sankhya_options_set_int(co, "iteration_limit", 200000);
    sankhya_solution* cs = nullptr;
    const Route route;
    check(sankhya_solve(cm, co, &cs) == SANKHYA_OK, "C API: solve call");
    check(route.moved_by(1), "C API: the seam ran once");
    if (cs != nullptr) {
      std::vector<double> x(reference.col_value.size());
      sankhya_solution_col_values(cs, x.data(), static_cast<int>(x.size()));
      check(sankhya_solution_status(cs) == SANKHYA_OPTIMAL, "C API: optimal");
      check(sankhya_solution_iterations(cs) == reference.iterations, "C API: iterations");
      check(same(sankhya_solution_objective(cs), reference.objective), "C API: objective");
      check(same(x, reference.col_value), "C API: col_value");
      sankhya_solution_free(cs);
    }
    sankhya_options_free(co);
    sankhya_model_free(cm);
  }

  // 7. The banner reports the device through the seam's probe.
  check(std::string(sankhya::banner()).find("GB300 (stand-in)") != std::string::npos,
        std::string("banner names the device: ") + sankhya::banner());

  // 8. Two virtual devices on device 0.
  {
    sankhya::Options o;
    o.set_bool("log_to_console", false);
    o.set_double("pdhg_tolerance", 1e-6);
    o.set_bool("pdhg_polish", false);
    o.set_int("iteration_limit", 500000);
    sankhya::Logger silent(nullptr);
    const sankhya::Solution single = sankhya::gpu::solve_pdhg_gpu(model, o, silent);
    const sankhya::Solution multi = sankhya::gpu::solve_pdhg_multi_gpu(model, o, {0, 0}, silent);
    check(single.status == sankhya::SolveStatus::kOptimal, "virtual devices: single optimal");
    check(multi.status == sankhya::SolveStatus::kOptimal, "virtual devices: multi optimal");
    check(std::fabs(multi.objective - single.objective) <=
              1e-5 * std::max(1.0, std::fabs(single.objective)),
          "virtual devices: the single-device objective");
    check(multi.algorithm == "pdhg-gpu", "virtual devices: one device (" + multi.algorithm + ")");
  }

  if (g_failures == 0) std::printf("OK\n");
  return g_failures == 0 ? 0 : 1;
}
