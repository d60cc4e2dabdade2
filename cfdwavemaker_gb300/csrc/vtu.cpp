// .vtu export of the s-grid ring.
//
// Follows lsGridSpline::write_vtk / export_vtu (oystelan/CFDwavemaker v3.1.0,
// src/lsgrid_spline.cpp:1200-1403): an ASCII VTK UnstructuredGrid of the nodes
// of one ring slot -- the base slot (tstep+1)%4 at t0, or with `last` the
// slot (tstep+2)%4 at t0+dt -- with the velocity as point data, the node
// positions (the level heights from that slot's elevation) as points, and
// hexahedra (quads for a grid that is flat in one direction) as cells.  The
// text is the reference's line for line; the values are the FP32 ring values.
//
// GB300 design: the slot is copied from HBM in one pass (16 B per node), and
// the text, about 100 B per node, is formatted by all host threads into
// per-thread buffers that are written in order.
#include "cfdwm.h"

#include <cuda_runtime.h>

#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

namespace cfdwm {

namespace {

// appends printf-formatted text to s
template <typename... A>
void app(std::string &s, const char *fmt, A... a) {
    char b[160];
    int n = std::snprintf(b, sizeof b, fmt, a...);
    if (n > 0) s.append(b, (size_t)std::min<int>(n, (int)sizeof b - 1));
}

// runs body(lo, hi, out) over [0, n) in ordered chunks on the host threads
// and concatenates the chunk outputs in order
template <typename F>
void parallel_text(long n, std::string &out, F body) {
    if (n <= 0) return;
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    long nt = std::min<long>(std::min<long>(hw, 64), std::max<long>(1, n / 64));
    std::vector<std::string> part((size_t)nt);
    std::vector<std::thread> th;
    for (long k = 0; k < nt; k++) {
        long lo = n * k / nt, hi = n * (k + 1) / nt;
        th.emplace_back([&, k, lo, hi] { body(lo, hi, part[(size_t)k]); });
    }
    for (auto &t : th) t.join();
    size_t tot = out.size();
    for (auto &p : part) tot += p.size();
    out.reserve(tot);
    for (auto &p : part) out += p;
}

int dir_exists(const char *path) {
    struct stat info;
    if (stat(path, &info) != 0) return (errno == ENOENT || errno == ENOTDIR) ? 0 : -1;
    return (info.st_mode & S_IFDIR) ? 1 : 0;
}

}  // namespace

int grid_write_vtu(const DevGrid &g, const std::string &path, const std::string &timelabel, bool last,
                   void *stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    const int nx = g.nx, ny = g.ny, nl = g.nl;
    if (nx < 1 || ny < 1 || nl < 1 || !g.ETA) return E_NOT_INITIALIZED;
    const int tt = last ? (g.tstep + 2) % 4 : (g.tstep + 1) % 4;
    const long c = (long)nx * ny, v = c * nl;
    std::vector<float> eta(c), U(3 * v);
    if (cudaMemcpyAsync(eta.data(), g.ETA + (long)tt * c, sizeof(float) * c, cudaMemcpyDeviceToHost, stream) !=
        cudaSuccess)
        return E_CUDA;
    for (int f = 0; f < 3; f++)
        if (cudaMemcpyAsync(U.data() + f * v, g.U[f] + (long)tt * v, sizeof(float) * v, cudaMemcpyDeviceToHost,
                            stream) != cudaSuccess)
            return E_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return E_CUDA;

    const double tval = last ? g.t0 + g.dt : g.t0;
    std::string s;
    s += "<?xml version=\"1.0\"?>\n"
         "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
    s += "\t <UnstructuredGrid>\n";
    s += "\t\t <FieldData> \n";
    app(s, "\t\t\t <DataArray type = \"Float64\" Name = \"%s\" NumberOfTuples = \"1\" format = \"ascii\" "
           "RangeMin = \"%.3f\" RangeMax = \"%.3f\"> \n",
        timelabel.c_str(), tval, tval);
    app(s, "\t\t\t %.3f \n", tval);
    s += "\t\t\t </DataArray > \n";
    s += "\t\t </FieldData> \n";
    app(s, "\t\t <Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", (int)v,
        std::max(nx - 1, 1) * std::max(ny - 1, 1) * std::max(nl - 1, 1));
    s += "\t\t\t <PointData Scalars=\"scalars\">\n";
    s += "\t\t\t\t <DataArray type=\"Float64\" NumberOfComponents=\"3\" Name=\"Velocity\" format=\"ascii\">\n";
    // node order i, j, m: the layout of the slot
    parallel_text(v, s, [&](long lo, long hi, std::string &o) {
        o.reserve((size_t)(hi - lo) * 40);
        for (long e = lo; e < hi; e++)
            app(o, "%g %g %g\n", (double)U[e], (double)U[v + e], (double)U[2 * v + e]);
    });
    s += "\t\t\t\t </DataArray>\n";
    s += "\t\t\t </PointData>\n";
    s += "\t\t\t <Points>\n";
    s += "\t\t\t\t <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
    const double x0 = g.cfg.domain[0], y0 = g.cfg.domain[2];
    const double ta = g.cfg.tan_a, tb = g.cfg.tan_b, h = g.depth, swl = g.swl;
    std::vector<double> lev(nl);   // s2tan(-1 + ds m), lsgrid_spline.cpp:100-104
    for (int m = 0; m < nl; m++) lev[m] = -std::pow(std::tan(-(-1. + g.ds * m) * ta), tb) / std::pow(std::tan(ta), tb);
    parallel_text(v, s, [&](long lo, long hi, std::string &o) {
        o.reserve((size_t)(hi - lo) * 40);
        for (long e = lo; e < hi; e++) {
            const long col = e / nl;
            const int m = (int)(e % nl), i = (int)(col / ny), j = (int)(col % ny);
            const double xpt = x0 + g.dx * i, ypt = y0 + g.dy * j, et = (double)eta[col];
            const double z = (et - swl) + lev[m] * (h + (et - swl));   // s2z, :96-98
            app(o, "%12.4f %12.4f %12.4f\n", xpt, ypt, z);
        }
    });
    s += "\t\t\t\t </DataArray>\n";
    s += "\t\t\t </Points>\n";
    s += "\t\t\t <Cells>\n";
    s += "\t\t\t\t <DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n";
    auto tail = [&](long ncell, int per, const char *type) {
        s += "\t\t\t\t </DataArray>\n";
        s += "\t\t\t\t <DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n";
        parallel_text(ncell, s, [&](long lo, long hi, std::string &o) {
            for (long q = lo; q < hi; q++) app(o, "%d \n", (int)((q + 1) * per));
        });
        s += "\t\t\t\t </DataArray>\n";
        s += "\t\t\t\t <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
        std::string ty = std::string(type) + " \n";
        s.reserve(s.size() + (size_t)ncell * ty.size());
        for (long q = 0; q < ncell; q++) s += ty;
    };
    if (nx > 1 && ny > 1 && nl > 1) {
        const long ncell = (long)(nx - 1) * (ny - 1) * (nl - 1);
        parallel_text(ncell, s, [&](long lo, long hi, std::string &o) {
            for (long q = lo; q < hi; q++) {
                const int m = (int)(q % (nl - 1)), j = (int)((q / (nl - 1)) % (ny - 1)),
                          i = (int)(q / ((long)(nl - 1) * (ny - 1)));
                const unsigned a1 = nl * ny * i + nl * j + m, a2 = nl * ny * (i + 1) + nl * j + m;
                const unsigned a3 = nl * ny * (i + 1) + nl * (j + 1) + m, a4 = nl * ny * i + nl * (j + 1) + m;
                app(o, "%u %u %u %u %u %u %u %u\n", a1, a2, a3, a4, a1 + 1, a2 + 1, a3 + 1, a4 + 1);
            }
        });
        tail(ncell, 8, "12");
    } else if (nx > 1 && ny == 1 && nl > 1) {
        const long ncell = (long)(nx - 1) * (nl - 1);
        for (int i = 0; i < nx - 1; i++)
            for (int m = 0; m < nl - 1; m++)
                app(s, "%u %u %u %u\n", (unsigned)(nl * i + m), (unsigned)(nl * (i + 1) + m),
                    (unsigned)(nl * (i + 1) + m + 1), (unsigned)(nl * i + m + 1));
        tail(ncell, 4, "9");
    } else if (nx == 1 && ny > 1 && nl > 1) {
        const long ncell = (long)(ny - 1) * (nl - 1);
        for (int j = 0; j < ny - 1; j++)
            for (int m = 0; m < nl - 1; m++)
                app(s, "%u %u %u %u\n", (unsigned)(nl * j + m), (unsigned)(nl * (j + 1) + m),
                    (unsigned)(nl * (j + 1) + m + 1), (unsigned)(nl * j + m + 1));
        tail(ncell, 4, "9");
    } else if (nx > 1 && ny > 1 && nl == 1) {
        const long ncell = (long)(nx - 1) * (ny - 1);
        for (int i = 0; i < nx - 1; i++)
            for (int j = 0; j < ny - 1; j++)
                app(s, "%u %u %u %u\n", (unsigned)(ny * i + j), (unsigned)(ny * (i + 1) + j),
                    (unsigned)(ny * (i + 1) + j + 1), (unsigned)(ny * i + j + 1));
        tail(ncell, 4, "9");
    }
    s += "\t\t\t\t </DataArray>\n";
    s += "\t\t\t </Cells>\n";
    s += "\t\t </Piece>\n";
    s += "\t </UnstructuredGrid>\n";
    s += "</VTKFile>\n";
    FILE *fp = std::fopen(path.c_str(), "w");
    if (!fp) return E_NO_FILE;
    bool ok = std::fwrite(s.data(), 1, s.size(), fp) == s.size();
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? OK : E_NO_FILE;
}

int grid_dump_vtu(const DevGrid &g, bool last, void *stream) {
    const LsgridCfg &c = g.cfg;
    if (dir_exists(c.vtk_path.c_str()) == 0) {
        std::fprintf(stderr,
                     "WARNING: Specified directory for storage of VTK files does not exist. Directory will be "
                     "created at the following path:  %s\n",
                     c.vtk_path.c_str());
        mkdir(c.vtk_path.c_str(), 0755);
    }
    char buf[32];
    std::snprintf(buf, sizeof buf, "%05d", g.tstep);
    return grid_write_vtu(g, c.vtk_path + c.vtk_prefix + buf + ".vtu", c.vtk_timelabel, last, stream);
}

}  // namespace cfdwm
