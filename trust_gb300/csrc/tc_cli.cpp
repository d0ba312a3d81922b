// tc_cli.cpp — command-line program with the reference's argv and output line.
//
//   trust_tc <folder> <nGPUs> <threads> <blocks> <chunk>          (Without-graph-partition/mpi_main.cpp:75-119)
//   trust_tc <folder> <nGPUs> <threads> <blocks> <chunk> <n>      (With-graph-partition/mpi_main.cpp:75-127)
//
// Logical ranks are looped as the reference does when fewer processes than ranks run
// (Without-graph-partition/mpi_main.cpp:94-104); on one GPU rank 0 carries the whole count.  Output, unchanged:
//   "%s,%d,%d,%lld,%f,%f \n"  folder, vertices, edges, triangles, max time, GTEPS   (W main :115)
//   "\n%s,triangle:%lld,%f,%f\n" folder, triangles, min time, max time            (P main :123)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/trust_tc.h"
#include "../../include/trust_tc_shim.h"

static void usage(const char *prog) {
  fprintf(stderr, "usage: %s <folder> <nGPUs> <threads> <blocks> <chunk> [partitions]\n",
          prog);
}

int main(int argc, char *argv[]) {
  int npos = 0;
  const char *pos[7] = {0};
  for (int i = 1; i < argc; ++i) {
    if (strncmp(argv[i], "--", 2) == 0) {
      usage(argv[0]);
      return 2;
    }
    if (npos < 6) pos[npos] = argv[i];
    ++npos;
  }
  if (npos != 5 && npos != 6) {
    usage(argv[0]);
    return 2;
  }
  char name[4096];
  snprintf(name, sizeof name, "%s", pos[0]);
  const int total_rank = atoi(pos[1]), threads = atoi(pos[2]), blocks = atoi(pos[3]), chunk = atoi(pos[4]);
  if (total_rank < 1 || threads < 0 || blocks < 0 || chunk < 0) {
    usage(argv[0]);
    return 2;
  }
  const int partitioned = npos == 6;
  const int parts = partitioned ? atoi(pos[5]) : 0;
  if (partitioned && parts < 1) {
    usage(argv[0]);
    return 2;
  }
  struct arguments args = {0, 0, 0.0, 0, 0};
  long long sum = 0;
  double tmin = 9999, tmax = 0;
  for (int rank = 0; rank < total_rank; ++rank) {
    if (partitioned)
      args = Triangle_count(rank, name, args, total_rank, threads, blocks, chunk, parts);
    else
      args = Triangle_count(rank, name, args, total_rank, threads, blocks, chunk);
    if (rank == 0 || args.time > 0) {
      if (tmin > args.time) tmin = args.time;
      if (tmax < args.time) tmax = args.time;
    }
    sum += args.count;
  }
  if (partitioned)
    printf("\n%s,triangle:%lld,%f,%f\n", pos[0], sum, tmin, tmax);
  else
    printf("%s,%d,%d,%lld,%f,%f \n", pos[0], args.vertices, args.edge_count, sum, tmax,
           (args.edge_count / tmax / 1000000000));
  return 0;
}
