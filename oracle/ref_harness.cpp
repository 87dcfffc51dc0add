// ref_harness.cpp -- C entry points around the reference's own CPU classes
// (TEST INFRASTRUCTURE ONLY).  Linked with the reference's cpu_toed.cpp and
// subpix_TO_correction/subpix_to_correction.cpp, compiled where they lie by
// oracle/Makefile into oracle/_ref/libref_toed.so.  Used to pin the oracle
// restatement (oracle/toed_oracle.c) and to generate tests/golden fixtures.
//
// The detector class reads the image through preprocessing(std::ifstream&)
// (cpu_toed.cpp:97-126), one byte per pixel with get().  The harness writes
// a header-less byte stream to a scratch file, so the raw-PGM header quirk of
// main_cpu_DP.cpp:162 does not apply.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <math.h>
#include <omp.h>
#include <string.h>
#include <string>
#include <vector>

#include <algorithm>
#include <unordered_map>

#include <fcntl.h>
#include <unistd.h>

// Read access to the intermediate planes for plane-level pinning (both
// classes keep them in their implicit private sections).
#define class struct
#define private public
#include "cpu_toed.hpp"
#include "subpix_to_correction.hpp"
#undef private
#undef class

// The reference classes print progress lines to stdout; each entry point
// sends them to /dev/null so that a caller's own stdout stays parseable.
namespace {
struct QuietStdout {
    int saved = -1;
    QuietStdout()
    {
        std::fflush(stdout);
        std::cout.flush();
        saved = dup(1);
        const int nul = open("/dev/null", O_WRONLY);
        if (nul >= 0) {
            dup2(nul, 1);
            close(nul);
        }
    }
    ~QuietStdout()
    {
        std::fflush(stdout);
        std::cout.flush();
        if (saved >= 0) {
            dup2(saved, 1);
            close(saved);
        }
    }
};
}  // namespace

extern "C" {

// TOED, FP64, sigma = 2 / kernel 17 (the reference's fixed configuration,
// main_cpu_DP.cpp:182-183).  img: H*W bytes.  edges: capacity*4 doubles.
// planes4 (optional): Ix, Iy, |grad|, orientation, each (2H)(2W).
// posmaps (optional): subpix_pos_x, subpix_pos_y, subpix strength.
// Returns N (edgels written: min(N, capacity)), or -1 on IO error.
long ref_toed_detect_u8(const unsigned char* img, int H, int W, int nthreads,
                        const char* scratch_dir, double* edges, long capacity,
                        double* planes4, double* posmaps, double* time_conv_nms)
{
    QuietStdout quiet;
    std::string dir(scratch_dir ? scratch_dir : ".");
    std::string path = dir + "/ref_input.bin";
    {
        std::ofstream f(path, std::ios::binary);
        if (!f.is_open()) return -1;
        f.write(reinterpret_cast<const char*>(img), (std::streamsize)H * W);
    }
    std::ifstream in(path, std::ios::binary);
    if (!in.is_open()) return -1;

    ThirdOrderEdgeDetectionCPU<double> det(H, W, 2, 17, nthreads);
    det.set_output_dir(dir);
    det.preprocessing(in);
    det.convolve_img();
    std::vector<double> buf((size_t)(2 * H) * (2 * W) * 4, 0.0);
    int N = det.non_maximum_suppresion(buf.data());
    long nw = N < capacity ? N : capacity;
    if (nw > 0) std::memcpy(edges, buf.data(), sizeof(double) * 4 * nw);
    const size_t P2 = (size_t)(2 * H) * (2 * W);
    if (planes4) {
        std::memcpy(planes4 + 0 * P2, det.Ix, sizeof(double) * P2);
        std::memcpy(planes4 + 1 * P2, det.Iy, sizeof(double) * P2);
        std::memcpy(planes4 + 2 * P2, det.I_grad_mag, sizeof(double) * P2);
        std::memcpy(planes4 + 3 * P2, det.I_orient, sizeof(double) * P2);
    }
    if (posmaps) {
        std::memcpy(posmaps + 0 * P2, det.subpix_pos_x_map, sizeof(double) * P2);
        std::memcpy(posmaps + 1 * P2, det.subpix_pos_y_map, sizeof(double) * P2);
        std::memcpy(posmaps + 2 * P2, det.subpix_grad_mag_map, sizeof(double) * P2);
    }
    if (time_conv_nms) {
        time_conv_nms[0] = det.time_conv;
        time_conv_nms[1] = det.time_nms;
    }
    std::remove(path.c_str());
    return N;
}

// Subpixel TO correction, FP64, interp_n = 0 (main_subpix_to_correction.cpp:279-293).
// theta: optional h*w orientation; NULL -> estimate_orientation().
// TO_E / TO_O: optional dense outputs.  times: optional [nms, conv, correct, orient].
long ref_subpix_to_correct(const double* E, int h, int w, double thresh, double sigma,
                           int nthreads, double nbr_radius, const double* theta,
                           const char* scratch_dir, double* edges, long capacity,
                           double* TO_E, double* TO_O, double* theta_out, double* times)
{
    QuietStdout quiet;
    SubpixelTOCorrectionCPU<double> tc(h, w, thresh, sigma, nthreads, 0);
    tc.set_output_dir(scratch_dir ? scratch_dir : ".");
    tc.set_neighbor_radius(nbr_radius);
    tc.set_edgemap(E);
    double t_or = 0;
    if (theta) {
        tc.set_orientation(theta);
    } else {
        double t0 = omp_get_wtime();
        tc.estimate_orientation();
        t_or = omp_get_wtime() - t0;
    }
    if (theta_out) std::memcpy(theta_out, tc.theta, sizeof(double) * (size_t)h * w);
    std::vector<double> buf((size_t)h * w * 4, 0.0);
    int N = tc.run(buf.data());
    long nw = N < capacity ? N : capacity;
    if (nw > 0) std::memcpy(edges, buf.data(), sizeof(double) * 4 * nw);
    if (TO_E) std::memcpy(TO_E, tc.TO_edgemap, sizeof(double) * (size_t)h * w);
    if (TO_O) std::memcpy(TO_O, tc.TO_orientation, sizeof(double) * (size_t)h * w);
    if (times) {
        times[0] = tc.time_nms;
        times[1] = tc.time_conv;
        times[2] = tc.time_correct;
        times[3] = t_or;
    }
    return N;
}

// The same at interp_n >= 0 (the map resized onto the 2^n work grid by the
// class itself, set_edgemap :224-233).  TO_E / TO_O: optional, h*w.
long ref_subpix_to_correct_n(const double* E, int h, int w, int interp_n, double thresh, double sigma,
                             int nthreads, double nbr_radius, const double* theta, const char* scratch_dir,
                             double* edges, long capacity, double* TO_E, double* TO_O)
{
    QuietStdout quiet;
    SubpixelTOCorrectionCPU<double> tc(h, w, thresh, sigma, nthreads, interp_n);
    tc.set_output_dir(scratch_dir ? scratch_dir : ".");
    tc.set_neighbor_radius(nbr_radius);
    tc.set_edgemap(E);
    if (theta)
        tc.set_orientation(theta);
    else
        tc.estimate_orientation();
    std::vector<double> buf((size_t)tc.work_height * tc.work_width * 4, 0.0);
    int N = tc.run(buf.data());
    long nw = N < capacity ? N : capacity;
    if (nw > 0) std::memcpy(edges, buf.data(), sizeof(double) * 4 * nw);
    if (TO_E) std::memcpy(TO_E, tc.TO_edgemap, sizeof(double) * (size_t)h * w);
    if (TO_O) std::memcpy(TO_O, tc.TO_orientation, sizeof(double) * (size_t)h * w);
    return N;
}

}  // extern "C"
