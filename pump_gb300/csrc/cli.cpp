// `pump <input file> <cp target> <eta>` -- the reference's command line
// (mainPUMP.cu:82-111, README.md:5-9) over libpump.
//
// The sample count, a compile-time NUM in the reference (Makefile:1-5), is
// read from the environment variable PUMP_NUM (default 1000).  Optional
// flags after the three positional arguments: --num N, --disc D (edge
// discretisation), --particles P (HSMC particles), --precision (closed-form
// binary64 BVP instead of the reference's bisection), --gpu-arith (the pair
// BVPs in the arithmetic of the reference's own GPU kernel, PUMP_BVP_PARITY_GPU;
// by default the parity arithmetic of the reference's host code), --seed S.
// Writes path.txt like PUMP.cu:591-594 when a solution is found and
// discretizedPath.txt like PUMP.cu:571-579 whenever the search ran, and
// prints the reference's final summary lines (PUMP.cu:582-604).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

#include "pump.h"

int main(int argc, char **argv) {
  if (argc < 4) {
    std::cout << "Must specify an online setting filename, i.e. $ ./pump <file.txt> <cp target> <cp factor>"
              << std::endl;
    return EXIT_FAILURE;
  }
  pump_problem pb;
  pump_problem_defaults(&pb);
  const char *env_num = std::getenv("PUMP_NUM");
  if (env_num) pb.N = std::atoi(env_num);
  for (int a = 4; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--num") && a + 1 < argc) pb.N = std::atoi(argv[++a]);
    else if (!std::strcmp(argv[a], "--disc") && a + 1 < argc) pb.num_disc = std::atoi(argv[++a]);
    else if (!std::strcmp(argv[a], "--particles") && a + 1 < argc) pb.num_hsmc = std::atoi(argv[++a]);
    else if (!std::strcmp(argv[a], "--seed") && a + 1 < argc) pb.seed = std::strtoull(argv[++a], nullptr, 0);
    else if (!std::strcmp(argv[a], "--precision")) pb.bvp_mode = PUMP_BVP_PRECISION;
    else if (!std::strcmp(argv[a], "--gpu-arith")) pb.bvp_mode = PUMP_BVP_PARITY_GPU;
  }
  pb.cp_target = (float)std::atof(argv[2]);
  pb.cp_factor = (float)std::atof(argv[3]);
  if (pump_read_input(argv[1], &pb) != PUMP_OK)
    std::cout << "file ain't good, keeping set parameters" << std::endl << std::endl;

  pump_ctx *ctx = nullptr;
  pump_status_t st = pump_ctx_create(0, &ctx);
  if (st != PUMP_OK) {
    std::cerr << "pump: " << pump_status_string(st) << ": " << pump_last_error() << std::endl;
    return EXIT_FAILURE;
  }
  std::vector<float> path((size_t)pb.table_rows * PUMP_DIM);
  std::vector<int> nodes(64);
  std::vector<float> ctrl((size_t)8192 * PUMP_DIM);
  pump_plan_result res;
  std::memset(&res, 0, sizeof res);
  res.path = path.data();
  res.path_cap = pb.table_rows;
  res.nodes = nodes.data();
  res.nodes_cap = (int)nodes.size();
  res.ctrl_path = ctrl.data();
  res.ctrl_cap = 8192;
  st = pump_plan(ctx, &pb, &res, nullptr);
  if (st == PUMP_OK || st == PUMP_ERR_NO_SOLUTION) {
    if (res.ctrl_len > res.ctrl_cap) {  // rare: plan again with room for every row
      ctrl.assign((size_t)res.ctrl_len * PUMP_DIM, 0.0f);
      res.ctrl_path = ctrl.data();
      res.ctrl_cap = res.ctrl_len;
      st = pump_plan(ctx, &pb, &res, nullptr);
    }
    std::ofstream cs("discretizedPath.txt");
    for (int i = 0; i < res.ctrl_len * PUMP_DIM; ++i) {
      cs << ctrl[i] << ", ";
      if ((i + 1) % PUMP_DIM == 0) cs << std::endl;
    }
  }
  std::cout << "number of goal paths found = " << res.goal_paths << " with a total number of paths = "
            << res.num_paths << " of " << res.num_considered << std::endl;
  std::cout << "****************** Final output ******************" << std::endl;
  if (st == PUMP_OK && res.success) {
    std::cout << "Search took: " << res.ms_search / 1000 << " s" << std::endl;
    std::cout << "Solution path = " << res.soln_path_idx << " with cp = " << res.soln_cp
              << " and cost = " << res.soln_cost << std::endl;
    std::cout << "nodes = [";
    for (int k = res.num_nodes - 1; k >= 0; --k)
      std::cout << nodes[k] << (k ? ", " : "");
    std::cout << "]" << std::endl;
    std::ofstream ofs("path.txt", std::ofstream::out);
    for (int i = 0; i < res.path_len; ++i) {
      for (int d = 0; d < PUMP_DIM; ++d) ofs << path[(size_t)i * PUMP_DIM + d] << " ";
      ofs << std::endl;
    }
  } else if (st == PUMP_OK || st == PUMP_ERR_NO_SOLUTION) {
    std::cout << "FAILURE, need to restart search" << std::endl;
  } else {
    std::cerr << "pump: " << pump_status_string(st) << ": " << pump_last_error() << std::endl;
  }
  std::cout << "****************** To Excel results: ******************" << std::endl;
  std::cout << "cp: \t\t\t" << res.soln_cp << std::endl;
  std::cout << "cost: \t\t\t" << res.soln_cost << std::endl;
  std::cout << "Roadmap time: \t\t" << res.ms_roadmap << " ms" << std::endl;
  std::cout << "Online time: \t\t" << res.ms_online << " ms" << std::endl;
  std::cout << "Explore time: \t\t" << res.ms_explore << " ms" << std::endl;
  std::cout << "SolnSearch time: \t" << res.ms_search << " ms" << std::endl;
  pump_ctx_destroy(ctx);
  return (st == PUMP_OK || st == PUMP_ERR_NO_SOLUTION) ? EXIT_SUCCESS : EXIT_FAILURE;
}
