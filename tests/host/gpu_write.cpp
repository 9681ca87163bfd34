// gpu_write.cpp -- one model solved by SANKHYA's solve() on the GB300 engine, written out for
// the reference's independent verifier.
//
// Linked with the reference's whole core (solve(), the readers, the writer; oracle/Makefile
// `ref-core`), the seam files that replace src/gpu and the engine's real library
// (lib/libsankhya_gb300.so): the path a maintainer ships, with no stand-in anywhere.
// `gpu_write model.mps out.sol [tolerance]` solves the model with algorithm=pdhg, gpu=true
// (tolerance 1e-8 unless given, no interior-point polish) and writes the answer with
// io::write_solution (src/io/writer.cpp), which tools/verify_solution.py reads. It exits 1 unless the answer came
// through the seam ("pdhg-gpu"), 2 when the model cannot be read or the answer written.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "sankhya/io.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"

int main(int argc, char** argv) {
  if (argc < 3 || argc > 4) {
    std::printf("usage: gpu_write model.mps out.sol [tolerance]\n");
    return 2;
  }
  sankhya::Model model;
  const sankhya::io::ReadResult read = sankhya::io::read_model(argv[1], &model);
  if (!read.ok) {
    std::printf("cannot read %s: %s\n", argv[1], read.error.c_str());
    return 2;
  }
  sankhya::Options o;
  o.set_bool("log_to_console", false);
  o.set_string("algorithm", "pdhg");
  o.set_bool("gpu", true);
  o.set_bool("pdhg_polish", false);
  o.set_double("pdhg_tolerance", argc >= 4 ? std::atof(argv[3]) : 1e-8);
  o.set_int("iteration_limit", 1000000);
  const sankhya::Solution s = sankhya::solve(model, o);
  std::string error;
  if (!sankhya::io::write_solution(argv[2], model, s, o, &error)) {
    std::printf("cannot write %s: %s\n", argv[2], error.c_str());
    return 2;
  }
  std::printf("%s: %s, %lld iterations, objective %.17g, algorithm %s\n", argv[1],
              sankhya::to_string(s.status), static_cast<long long>(s.iterations), s.objective,
              s.algorithm.c_str());
  if (!s.message.empty()) std::printf("%s\n", s.message.c_str());
  return s.algorithm == "pdhg-gpu" ? 0 : 1;
}
