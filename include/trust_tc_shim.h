/*
 * trust_tc_shim.h — the reference's C++ operator signature over the C ABI.
 *
 * Declares the same `struct arguments` and `Triangle_count` as Without-graph-partition/TC.cuh:2-10
 * (C++ linkage), plus the partitioned overload of With-graph-partition/TC.cuh:10, so a non-MPI
 * main program written like Without-graph-partition/mpi_main.cpp:75-119 links against
 * libtrust_tc.so unchanged.  Error behaviour matches the reference's HRR macro (Without-graph-partition/
 * herror.h:1-8): the message is printed and the process exits with EXIT_FAILURE.  Logical ranks:
 * the library counts on one GPU, so rank 0 returns the whole count and ranks > 0 return 0 (the
 * main program's SUM over ranks, Without-graph-partition/mpi_main.cpp:110-112, is unchanged).
 */
#ifndef TRUST_TC_SHIM_H
#define TRUST_TC_SHIM_H

struct arguments {
  int edge_count;
  long long count;
  double time;
  int degree;
  int vertices;
};

struct arguments Triangle_count(int rank, char name[100], struct arguments args, int total_process, int n_threads,
                                int n_blocks, int chunk_size);

struct arguments Triangle_count(int rank, char name[100], struct arguments args, int total_process, int n_threads,
                                int n_blocks, int chunk_size, int partition_num);

#endif
