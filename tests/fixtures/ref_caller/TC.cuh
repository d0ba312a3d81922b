// Test fixture: the declarations a TRUST main program sees through its own TC.cuh
// (Without-graph-partition/TC.cuh:1-10) - the `arguments` record and the operator's C++ signature.
// Only the interface is restated here; the definition comes from libtrust_tc.so at link time.

struct arguments{
    int edge_count;
    long long count;
    double time;
    int degree;
    int vertices;
};

struct arguments Triangle_count(int rank, char input[100], struct arguments args,int total_process, int threads, int blocks, int chunk_size);
