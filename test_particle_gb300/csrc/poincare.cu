// poincare.cu -- the Poincare map of the gridded magnetic field
// (src/poincare_map.c): seed points on a plane, field lines traced on the GPU
// (one thread per seed, track_fp64.cu), crossings of the plane recorded.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/tp_gpu.h"
#include "../../include/tp_h5.h"
#include "tp_internal.h"
#include "tp_kernels.h"

using namespace tp;

// The configuration globals of src/poincare_map.c:22-33.
extern "C" {
int map_for_single_point;
int face_cross_section;
int nhorizontal;
int nvertical;
int ncross;
double fx0, fy0, fz0;
double min_horizontal, max_horizontal;
double min_vertical, max_vertical;
double step_fieldline, fieldline_length_max;
}

extern "C" int tp_poincare_trace(int n, const double* seeds, int face, double step, double length_max,
                                 int nc, double* xpos, double* ypos, double* zpos, int* found)
{
    if (system_type != TP_SYS_MHD && system_type != TP_SYS_PIC) {
        set_error(6, "Poincare maps trace the gridded magnetic field (system types 3 and 4; got %d)",
                  system_type);
        return -1;
    }
    // (crossings per seed up to 2^24: the rows of nc + 1 entries are indexed
    // with 32-bit counts)
    if (n < 0 || face < 0 || face > 2 || !(step > 0.0) || !(length_max > 0.0) || nc < 1 || nc > (1 << 24) ||
        length_max / step > 2147483647.0) {
        set_error(6, "bad Poincare map arguments: n %d face %d step %g length %g crossings %d", n, face,
                  step, length_max, nc);
        return -1;
    }
    DevField f;
    if (!build_field(system_type, f)) return -1;
    if (!f.bc_f) {
        set_error(6, "Poincare map: no float magnetic field grid is set");
        return -1;
    }
    if (n == 0) return 0;
    const size_t row = (size_t)n * (nc + 1);
    double *d_seeds = nullptr, *d_out = nullptr;
    int* d_found = nullptr;
    bool ok = cuda_ok(cudaMalloc(&d_seeds, sizeof(double) * 3 * n), "seeds") &&
              cuda_ok(cudaMalloc(&d_out, sizeof(double) * 3 * row), "crossings") &&
              cuda_ok(cudaMalloc(&d_found, sizeof(int) * n), "found");
    cudaStream_t s = g.stream;
    if (ok) {
        cudaMemcpyAsync(d_seeds, seeds, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
        ok = cuda_ok(fp64::launch_poincare(f, n, d_seeds, face, step, length_max, nc, d_out, d_out + row,
                                           d_out + 2 * row, d_found, g.d_status, s),
                     "poincare");
    }
    if (ok) {
        cudaMemcpyAsync(xpos, d_out, sizeof(double) * row, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(ypos, d_out + row, sizeof(double) * row, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(zpos, d_out + 2 * row, sizeof(double) * row, cudaMemcpyDeviceToHost, s);
        if (found) cudaMemcpyAsync(found, d_found, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
        ok = cuda_ok(cudaStreamSynchronize(s), "poincare sync");
    }
    if (d_seeds) cudaFree(d_seeds);
    if (d_out) cudaFree(d_out);
    if (d_found) cudaFree(d_found);
    return ok ? 0 : -1;
}

// Default output of poincare_map when the caller provides none: the
// reference's data/poincare_map.h5 (src/poincare_map.c:185-235), group
// /poincare_map, datasets xpos, ypos, zpos [points][ncross + 1] of native
// doubles, each rank writing its rows (tp_h5_write_poincare, no libhdf5).  A
// caller may define this function to write the points elsewhere.
extern "C" __attribute__((weak)) void tp_poincare_save(int mpi_rank, int mpi_size, int npoints_total,
                                                       int nc, int nshift, int npoints, const double* xpos,
                                                       const double* ypos, const double* zpos)
{
    (void)mpi_rank;
    (void)mpi_size;
    if (tp_h5_write_poincare("data/poincare_map.h5", npoints_total, nc, nshift, npoints, xpos, ypos, zpos) != 0) {
        printf("ERROR: %s\n", tp_last_error());
        exit(1);
    }
}

// config_poincare_map, src/poincare_map.c:327-450 (same labels and order)
static void read_poincare_config(int mpi_rank, const char* config_file_name)
{
    FILE* fp = fopen(config_file_name, "r");
    if (!fp) {
        printf("Failed to open %s.\n", config_file_name);
        exit(1);
    }
    char buff[1024];
    while (fgets(buff, sizeof(buff), fp) != NULL)
        if (strstr(buff, "Poincare map configuration") != NULL) break;
    auto need = [&](int got, const char* what) {
        if (got != 1) {
            printf("Failed to get %s.\n", what);
            exit(1);
        }
    };
    need(fscanf(fp, "Which face as the cross section (0: x, 1: y, 2:z):%d\n", &face_cross_section),
         "the face for cross section");
    if (face_cross_section < 0 || face_cross_section > 2) {
        printf("ERROR: wrong face for cross section.");
        exit(1);
    }
    need(fscanf(fp, "Field-line tracking step: %lf\n", &step_fieldline), "the step for field-line tracking");
    need(fscanf(fp, "Maximum tracking length: %lf\n", &fieldline_length_max),
         "the maximum length for field-line tracking");
    need(fscanf(fp, "Number of crossing points: %d\n", &ncross), "the number of crossing points");
    map_for_single_point = 1;
    need(fscanf(fp, "Whether to get the map only for a single point:%d\n", &map_for_single_point),
         "flag for whether to get the map for only a single point");
    need(fscanf(fp, "x-position of the point: %lf\n", &fx0), "the x-position of the point");
    need(fscanf(fp, "y-position of the point: %lf\n", &fy0), "the y-position of the point");
    need(fscanf(fp, "z-position of the point: %lf\n", &fz0), "the z-position of the point");
    if (!map_for_single_point) {
        while (fgets(buff, sizeof(buff), fp) != NULL)
            if (strstr(buff, "for a 2D plane") != NULL) break;
        need(fscanf(fp, "min_horizontal: %lf\n", &min_horizontal), "min_horizontal");
        need(fscanf(fp, "max_horizontal: %lf\n", &max_horizontal), "max_horizontal");
        need(fscanf(fp, "min_vertical: %lf\n", &min_vertical), "min_vertical");
        need(fscanf(fp, "max_vertical: %lf\n", &max_vertical), "max_vertical");
        need(fscanf(fp, "nhorizontal: %d\n", &nhorizontal), "nhorizontal");
        need(fscanf(fp, "nvertical: %d\n", &nvertical), "nvertical");
    }
    fclose(fp);
    if (mpi_rank == 0) {
        printf("The step for field-line tracking: %lf\n", step_fieldline);
        printf("The maximum length for field-line tracking: %lf\n", fieldline_length_max);
        printf("Number of crossing points: %d\n", ncross);
    }
}

// src/poincare_map.c:39-239: seeds of this rank (the single point, or this
// rank's share of the nhorizontal x nvertical plane, split as the reference
// does), traced on the GPU, written by tp_poincare_save.
extern "C" int poincare_map(int mpi_rank, int mpi_size, char* config_file_name, domain* sdomain)
{
    if (mpi_rank == 0) printf("***** Entering Poincare *****\n");
    memcpy(&simul_domain, sdomain, sizeof(domain));
    read_poincare_config(mpi_rank, config_file_name);
    int npoints, nshift = 0, total;
    double* seeds;
    if (map_for_single_point) {
        npoints = total = 1;
        seeds = (double*)malloc(sizeof(double) * 3);
        seeds[0] = fx0; seeds[1] = fy0; seeds[2] = fz0;
    } else {
        total = nhorizontal * nvertical;
        npoints = total / mpi_size;
        nshift = npoints * mpi_rank;
        int res = total % mpi_size;
        if (res != 0) {
            if (mpi_rank < res) {
                npoints++;
                nshift += mpi_rank;
            } else {
                nshift += res;
            }
        }
        double dh = nhorizontal > 1 ? (max_horizontal - min_horizontal) / (nhorizontal - 1)
                                    : max_horizontal - min_horizontal;
        double dv = nvertical > 1 ? (max_vertical - min_vertical) / (nvertical - 1) : max_vertical - min_vertical;
        seeds = (double*)malloc(sizeof(double) * 3 * (npoints > 0 ? npoints : 1));
        for (int p = 0; p < npoints; p++) {
            int ip = nshift + p, iv = ip / nhorizontal, ih = ip % nhorizontal, count = 0;
            double* q = seeds + 3 * p;
            q[0] = fx0; q[1] = fy0; q[2] = fz0;
            for (int i = 0; i != 3; i++) {
                if (i == face_cross_section) continue;
                q[i] = count == 0 ? dh * ih + min_horizontal : dv * iv + min_vertical;
                count++;
            }
        }
    }
    size_t m = (size_t)(npoints > 0 ? npoints : 1) * (ncross + 1);
    double* xo = (double*)malloc(sizeof(double) * m);
    double* yo = (double*)malloc(sizeof(double) * m);
    double* zo = (double*)malloc(sizeof(double) * m);
    int* found = (int*)malloc(sizeof(int) * (npoints > 0 ? npoints : 1));
    if (tp_poincare_trace(npoints, seeds, face_cross_section, step_fieldline, fieldline_length_max, ncross, xo,
                          yo, zo, found) != 0)
        die_if_error("poincare_map");
    for (int p = 0; p < npoints; p++)
        if (found[p] < ncross)
            printf("Reached maximum length for field-line tracing before %d crosses\n", found[p] + 2);
    tp_poincare_save(mpi_rank, mpi_size, total, ncross, nshift, npoints, xo, yo, zo);
    free(seeds);
    free(xo);
    free(yo);
    free(zo);
    free(found);
    if (mpi_rank == 0) printf("***** Leaving Poincare *****\n");
    return 0;
}
