// Work-balanced contiguous partition of the s-grid's rows of columns over
// ranks (host code).
//
// The reference's MPI build gives rank r the rows [bounds[r], bounds[r+1]) of
// its grid, with per-row weights = the live (not ignored) columns of the row
// (lsgrid_spline.cpp:652-664) and the partition of mpi_utils.h:46-64.  The
// rule is kept exactly, so that a rank owns the same rows as the reference's
// rank of the same number:
//   * one rank, or no rows: everything on rank 0;
//   * all weights zero: the even split of mpi_utils.h:34-38 (the larger
//     blocks first);
//   * otherwise the rows are walked in order with a running weight sum acc,
//     and boundary r (1 <= r < s) is placed after the first row at which
//     acc * s >= r * total; at most one boundary is placed per row, so a
//     heavy row can push the next boundaries to later rows, and boundaries
//     never decrease.
#include "cfdwm.h"
#include "../../include/cfdwavemaker_gb300.h"

#include <algorithm>

namespace cfdwm {

void partition_columns(const long *w, int n, int nranks, int *bounds) {
    const int s = std::max(1, nranks);
    for (int r = 0; r < s; r++) bounds[r] = 0;
    bounds[s] = n;
    if (s == 1) return;
    long total = 0;
    for (int i = 0; i < n; i++) total += w[i];
    if (total <= 0) {
        const int chunk = n / s, rem = n % s;
        for (int r = 0; r < s; r++) bounds[r] = r * chunk + std::min(r, rem);
        bounds[s] = n;
        return;
    }
    long acc = 0;
    int r = 1;
    for (int i = 0; i < n && r < s; i++) {
        acc += w[i];
        if (acc * s >= (long)r * total) bounds[r++] = i + 1;
    }
    for (; r < s; r++) bounds[r] = n;
    for (int q = 1; q < s; q++) bounds[q] = std::max(bounds[q], bounds[q - 1]);
    bounds[s] = n;
}

}  // namespace cfdwm

extern "C" int cfdwm_partition_columns(const long *weights, int n, int nranks, int *bounds) {
    if (n < 0 || nranks < 1 || !bounds || (n > 0 && !weights)) return cfdwm::E_BAD_ARGUMENT;
    for (int i = 0; i < n; i++)
        if (weights[i] < 0) return cfdwm::E_BAD_ARGUMENT;
    cfdwm::partition_columns(weights, n, nranks, bounds);
    return cfdwm::OK;
}
