// Test fixture: a non-MPI main program that uses the operator the way
// Without-graph-partition/mpi_main.cpp:75-119 does for one process: argv = folder, logical ranks,
// threads, blocks, chunk; every logical rank is counted in turn, the counts are summed, and the
// reference's output line is printed (format of mpi_main.cpp:115).  It includes TC.cuh, not any
// header of this library, and is linked against libtrust_tc.so.
#include <stdio.h>
#include <stdlib.h>

#include "TC.cuh"

int main(int argc, char *argv[]) {
  if (argc != 6) return 2;
  const int total_rank = atoi(argv[2]), threads = atoi(argv[3]), blocks = atoi(argv[4]), chunk = atoi(argv[5]);
  struct arguments args = {0, 0, 0.0, 0, 0};
  long long sum = 0;
  double tmax = 0;
  for (int rank = 0; rank < total_rank; ++rank) {
    args = Triangle_count(rank, argv[1], args, total_rank, threads, blocks, chunk);
    if (tmax < args.time) tmax = args.time;
    sum += args.count;
  }
  printf("%s,%d,%d,%lld,%f,%f \n", argv[1], args.vertices, args.edge_count, sum, tmax,
         (args.edge_count / tmax / 1000000000));
  return 0;
}
