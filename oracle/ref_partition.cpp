// The reference's own column partition, compiled from its header
// (TEST INFRASTRUCTURE ONLY).
//
// mpi_utils.h (oystelan/CFDwavemaker v3.1.0 src/, unmodified) is included
// with MPI_enable set against the single-process stand-in oracle/mpi_stub/
// mpi.h, so cfdwm_mpi::partition_weighted (mpi_utils.h:46-64) runs as the
// reference's MPI build runs it for a communicator of `size` ranks.  Built
// by `make -C oracle ref` into oracle/_ref/; tests/test_shard_cpu.py pins the
// library's partition (cfdwm_partition_columns) against it.
#include <vector>

#include "mpi.h"
#define MPI_enable 1
#include "mpi_utils.h"

int refstub_size = 1;
int refstub_rank = 0;

extern "C" int refp_partition(const long *w, int n, int size, int *bounds) {
    refstub_size = size;
    std::vector<long> wv(w, w + n);
    std::vector<int> b;
    cfdwm_mpi::partition_weighted(wv, n, b);
    for (size_t q = 0; q < b.size(); q++) bounds[q] = b[q];
    return (int)b.size();
}
