// toed_gb300.hpp -- header-only C++ drop-in for the reference's GPU
// detection API, forwarding to the C ABI of toed_gb300.h.
//
// Mirrors (reference project paths):
//   template<typename T> class ThirdOrderEdgeDetectionGPU      gpu_toed.hpp:21-74
//     ctor (device, H, W, kernel_size, sigma)                  gpu_toed.hpp:79-135
//     preprocessing(std::ifstream&)                            gpu_toed.hpp:189-231
//     convolve_img()                                           gpu_toed.hpp:340-413
//     int non_maximum_suppresion(T* TOED_edges = nullptr)      gpu_toed.hpp:415-441
//     set_output_dir / write_array_to_file / read_array_from_file
//     public edge_pt_list_idx, num_of_edge_data, time_conv, time_nms, start, stop
//   void gpu_convolve(...) float / double                       gpu_kernels.hpp:24-45
//   void gpu_nms(...)      float / double                       gpu_kernels.hpp:48-63
//   template<typename T> class SubpixelTOCorrectionGPU, the GPU twin of
//     SubpixelTOCorrectionCPU<T>          subpix_TO_correction/subpix_to_correction.hpp:20-96
//     ctor (H, W, threshold, g_sigma, cpu_nthreads, n = 0), set_edgemap,
//     set_orientation, estimate_orientation, int run(T* edginfo_out),
//     set_output_dir, set_neighbor_radius, write_array_to_file; public
//     subpix_edge_pts_final, TO_edgemap, TO_orientation, edge_pt_list_idx,
//     num_of_edge_data, time_nms, time_conv, time_correct
//
// Differences a caller can see: convolve_img() runs the whole fused
// detection (convolution, NMS and ordering) and time_conv is its device time;
// non_maximum_suppresion() only copies the edgel list back (time_nms is that
// copy).  A sigma may be fractional (double overload).  Errors are printed and
// execution continues, as the reference's cudacheck does (gpu_kernels.hpp:10-17).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "toed_gb300.h"

namespace toed_shim {
inline void report(toed_status st, const char* what)
{
    if (st != TOED_OK)
        std::printf("\033[1;31mError in %s: %s %s\033[0m\n", what, toed_status_string(st),
                    st == TOED_ERR_CUDA ? toed_last_cuda_error() : "");
}
inline void report_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) std::printf("\033[1;31mError in %s: %s\033[0m\n", what, cudaGetErrorString(e));
}
}  // namespace toed_shim

template <typename T>
class ThirdOrderEdgeDetectionGPU {
    int device_id;
    int img_height;
    int img_width;
    int interp_img_height;
    int interp_img_width;
    int kernel_sz;
    double g_sig;
    std::string output_dir;
    toed_ctx* ctx = nullptr;
    std::vector<float> img;  // host copy of the input (FP32; uint8 values are exact)
    float* dev_img = nullptr;
    T* dev_edges = nullptr;
    int* dev_count = nullptr;
    int capacity = 0;
    std::vector<T> subpix_edge_pts_final;

    void init(int device, int H, int W, int kernel_size, double sigma)
    {
        device_id = device;
        img_height = H;
        img_width = W;
        interp_img_height = 2 * H;
        interp_img_width = 2 * W;
        kernel_sz = kernel_size;
        g_sig = sigma;
        output_dir = "./output_files";
        num_of_edge_data = 4;
        edge_pt_list_idx = 0;
        time_conv = time_nms = 0.f;
        img.assign((size_t)H * W, 0.f);
        // the reference sizes the edgel list for every 2x-grid point (main_gpu_cpu.cpp:57-66)
        capacity = interp_img_height * interp_img_width;
        toed_shim::report_cuda(cudaSetDevice(device), "cudaSetDevice");
        toed_shim::report(toed_create(&ctx, device), "toed_create");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_img, sizeof(float) * (size_t)H * W), "cudaMalloc");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_edges, sizeof(T) * 4 * (size_t)capacity), "cudaMalloc");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_count, sizeof(int)), "cudaMalloc");
        toed_shim::report_cuda(cudaEventCreate(&start), "cudaEventCreate");
        toed_shim::report_cuda(cudaEventCreate(&stop), "cudaEventCreate");
    }

  public:
    int edge_pt_list_idx;
    int num_of_edge_data;
    float time_conv, time_nms;
    cudaEvent_t start, stop;

    ThirdOrderEdgeDetectionGPU(int device, int H, int W, int kernel_size, int sigma)
    {
        init(device, H, W, kernel_size, (double)sigma);
    }
    ThirdOrderEdgeDetectionGPU(int device, int H, int W, int kernel_size, double sigma)
    {
        init(device, H, W, kernel_size, sigma);
    }
    ~ThirdOrderEdgeDetectionGPU()
    {
        cudaFree(dev_img);
        cudaFree(dev_edges);
        cudaFree(dev_count);
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        if (ctx) toed_destroy(ctx);
    }
    ThirdOrderEdgeDetectionGPU(const ThirdOrderEdgeDetectionGPU&) = delete;
    ThirdOrderEdgeDetectionGPU& operator=(const ThirdOrderEdgeDetectionGPU&) = delete;

    // One byte per pixel, as the reference reads it (gpu_toed.hpp:193-197).
    void preprocessing(std::ifstream& scan_infile)
    {
        for (int i = 0; i < img_height; i++)
            for (int j = 0; j < img_width; j++) img[(size_t)i * img_width + j] = (float)(int)scan_infile.get();
    }
    void preprocessing(const unsigned char* image)
    {
        for (size_t k = 0; k < img.size(); k++) img[k] = (float)image[k];
    }
    void preprocessing(const float* image) { std::memcpy(img.data(), image, sizeof(float) * img.size()); }

    void convolve_img()
    {
        toed_shim::report_cuda(cudaMemcpy(dev_img, img.data(), sizeof(float) * img.size(), cudaMemcpyHostToDevice),
                               "cudaMemcpy");
        toed_image im;
        im.pixels = dev_img;
        im.height = img_height;
        im.width = img_width;
        im.pitch = img_width;
        im.dtype = TOED_F32;
        im.edgels = dev_edges;
        im.capacity = capacity;
        im.count = dev_count;
        im.grid_index = nullptr;
        toed_params p;
        toed_params_default(&p, (float)g_sig);
        p.radius = (kernel_sz - 1) / 2;
        p.out_dtype = sizeof(T) == 8 ? TOED_F64 : TOED_F32;
        toed_shim::report_cuda(cudaEventRecord(start), "cudaEventRecord");
        toed_shim::report(toed_detect(ctx, &im, &p, 0), "toed_detect");
        toed_shim::report_cuda(cudaEventRecord(stop), "cudaEventRecord");
        toed_shim::report_cuda(cudaEventSynchronize(stop), "cudaEventSynchronize");
        toed_shim::report_cuda(cudaEventElapsedTime(&time_conv, start, stop), "cudaEventElapsedTime");
        std::printf(" ## GPU Convolution time = %8.4f ms\n", time_conv);
    }

    int non_maximum_suppresion(T* TOED_edges = nullptr)
    {
        toed_shim::report_cuda(cudaEventRecord(start), "cudaEventRecord");
        int n = 0;
        toed_shim::report_cuda(cudaMemcpy(&n, dev_count, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        const int m = n < capacity ? n : capacity;
        subpix_edge_pts_final.assign((size_t)4 * m, T(0));
        if (m > 0)
            toed_shim::report_cuda(cudaMemcpy(subpix_edge_pts_final.data(), dev_edges, sizeof(T) * 4 * (size_t)m,
                                              cudaMemcpyDeviceToHost),
                                   "cudaMemcpy");
        toed_shim::report_cuda(cudaEventRecord(stop), "cudaEventRecord");
        toed_shim::report_cuda(cudaEventSynchronize(stop), "cudaEventSynchronize");
        toed_shim::report_cuda(cudaEventElapsedTime(&time_nms, start, stop), "cudaEventElapsedTime");
        std::printf(" ## GPU NMS time = %8.4f ms\n", time_nms);
        if (TOED_edges != nullptr && m > 0) std::memcpy(TOED_edges, subpix_edge_pts_final.data(), sizeof(T) * 4 * (size_t)m);
        edge_pt_list_idx = m;
        write_array_to_file("data_final_output_gpu.txt", subpix_edge_pts_final.data(), m, num_of_edge_data);
        return m;
    }

    void set_output_dir(const std::string& dir) { output_dir = dir.empty() ? "./output_files" : dir; }

    // gpu_toed.hpp:452-478 (10 significant digits, tab separated)
    void write_array_to_file(std::string filename, T* wr_data, int first_dim, int second_dim)
    {
        std::cout << "writing data to a file " << filename << " ..." << std::endl;
        std::string out_file_name = output_dir;
        if (!out_file_name.empty() && out_file_name.back() != '/') out_file_name.push_back('/');
        out_file_name.append(filename);
        std::ofstream out_file(out_file_name);
        if (!out_file.is_open()) {
            std::cout << "write data file cannot be opened!" << std::endl;
            return;
        }
        out_file.precision(10);
        for (int i = 0; i < first_dim; i++) {
            for (int j = 0; j < second_dim; j++) out_file << wr_data[(size_t)i * second_dim + j] << "\t";
            out_file << "\n";
        }
    }

    // gpu_toed.hpp:483-509 (reads ./test_files/<name>)
    void read_array_from_file(std::string filename, T* rd_data, int first_dim, int second_dim)
    {
        std::ifstream in_file("./test_files/" + filename);
        if (!in_file) {
            std::cerr << "input read file not existed!\n";
            return;
        }
        T v;
        long long k = 0, n = (long long)first_dim * second_dim;
        while (k < n && (in_file >> v)) rd_data[k++] = v;
    }
};

namespace toed_shim {
template <typename T>
inline void convolve(int h, int w, T* dev_img, T* dev_Ix, T* dev_Iy, T* dev_I_grad_mag, T* dev_I_orient,
                     T* dev_Gx, T* dev_Gxx, T* dev_Gxxx, T* dev_G_of_x, T* dev_Gx_sh, T* dev_Gxx_sh, T* dev_Gxxx_sh,
                     T* dev_G_of_x_sh)
{
    // the reference kernel is built for 19-tap arrays (SHIFTED_KS = 19, gpu_convolve.cu:304-315)
    const int r = 8, n = 2 * r + 3;
    T* src[8] = {dev_G_of_x, dev_Gx, dev_Gxx, dev_Gxxx, dev_G_of_x_sh, dev_Gx_sh, dev_Gxx_sh, dev_Gxxx_sh};
    std::vector<T> tmp(n);
    std::vector<double> taps(8 * n);
    for (int f = 0; f < 8; ++f) {
        report_cuda(cudaMemcpy(tmp.data(), src[f], sizeof(T) * n, cudaMemcpyDeviceToHost), "cudaMemcpy");
        for (int k = 0; k < n; ++k) taps[f * n + k] = (double)tmp[k];
    }
    // TOED_GPU_CONVOLVE_DIRECT: the reference kernel's full 2-D window sums (its
    // FP32 rounding pattern) instead of the separable evaluation of the same planes
#ifdef TOED_GPU_CONVOLVE_DIRECT
    auto conv = toed_convolve_planes_direct;
#else
    auto conv = toed_convolve_planes;
#endif
    report(conv(dev_img, sizeof(T) == 8 ? TOED_F64 : TOED_F32, h, w, w, 2.0f, r, taps.data(),
                sizeof(T) == 8 ? TOED_F64 : TOED_F32, dev_Ix, dev_Iy, dev_I_grad_mag, dev_I_orient, 0),
           "gpu_convolve");
}
}  // namespace toed_shim

// gpu_kernels.hpp:24-45
inline void gpu_convolve(int device_id, int h, int w, int interp_h, int interp_w, float* dev_img, float* dev_Ix,
                         float* dev_Iy, float* dev_I_grad_mag, float* dev_I_orient, float* dev_Gx, float* dev_Gxx,
                         float* dev_Gxxx, float* dev_G_of_x, float* dev_Gx_sh, float* dev_Gxx_sh, float* dev_Gxxx_sh,
                         float* dev_G_of_x_sh)
{
    (void)device_id;
    (void)interp_h;
    (void)interp_w;
    toed_shim::convolve<float>(h, w, dev_img, dev_Ix, dev_Iy, dev_I_grad_mag, dev_I_orient, dev_Gx, dev_Gxx, dev_Gxxx,
                               dev_G_of_x, dev_Gx_sh, dev_Gxx_sh, dev_Gxxx_sh, dev_G_of_x_sh);
}
inline void gpu_convolve(int device_id, int h, int w, int interp_h, int interp_w, double* dev_img, double* dev_Ix,
                         double* dev_Iy, double* dev_I_grad_mag, double* dev_I_orient, double* dev_Gx,
                         double* dev_Gxx, double* dev_Gxxx, double* dev_G_of_x, double* dev_Gx_sh,
                         double* dev_Gxx_sh, double* dev_Gxxx_sh, double* dev_G_of_x_sh)
{
    (void)device_id;
    (void)interp_h;
    (void)interp_w;
    toed_shim::convolve<double>(h, w, dev_img, dev_Ix, dev_Iy, dev_I_grad_mag, dev_I_orient, dev_Gx, dev_Gxx,
                                dev_Gxxx, dev_G_of_x, dev_Gx_sh, dev_Gxx_sh, dev_Gxxx_sh, dev_G_of_x_sh);
}

// gpu_kernels.hpp:48-63 (threshold 2 and border 10 as gpu_nms.cu:97, :208)
inline void gpu_nms(int device_id, int interp_h, int interp_w, float* dev_Ix, float* dev_Iy, float* dev_I_grad_mag,
                    float* dev_subpix_pos_x_map, float* dev_subpix_pos_y_map)
{
    (void)device_id;
    toed_shim::report(toed_nms_planes(TOED_F32, interp_h, interp_w, dev_Ix, dev_Iy, dev_I_grad_mag, 2.0f, 10,
                                      dev_subpix_pos_x_map, dev_subpix_pos_y_map, 0),
                      "gpu_nms");
}
inline void gpu_nms(int device_id, int interp_h, int interp_w, double* dev_Ix, double* dev_Iy,
                    double* dev_I_grad_mag, double* dev_subpix_pos_x_map, double* dev_subpix_pos_y_map)
{
    (void)device_id;
    toed_shim::report(toed_nms_planes(TOED_F64, interp_h, interp_w, dev_Ix, dev_Iy, dev_I_grad_mag, 2.0f, 10,
                                      dev_subpix_pos_x_map, dev_subpix_pos_y_map, 0),
                      "gpu_nms");
}

// The subpixel third-order correction of a dense edge map, with the
// reference's SubpixelTOCorrectionCPU<T> interface, forwarding to
// toed_subpix_to_correct_batch.  Differences a caller can see: the orientation
// is estimated on the device inside run() when estimate_orientation() was
// called (or taken from set_orientation(), zeros until then, as the
// reference's theta buffer starts); cpu_nthreads is not used; time_conv holds
// the device time of the whole correction (NMS, convolutions and correction
// run as one pipeline), time_correct the copies of the results to the host,
// time_nms 0 (seconds, as the reference's omp_get_wtime differences).
template <typename T>
class SubpixelTOCorrectionGPU {
    int img_height, img_width, interp_n, work_height, work_width;
    T thresh, sigma, neighbor_radius;
    std::string output_dir;
    toed_ctx* ctx = nullptr;
    T* dev_E = nullptr;
    T* dev_theta = nullptr;
    bool estimate = false;
    T* dev_edges = nullptr;
    int* dev_count = nullptr;
    T* dev_TO_E = nullptr;
    T* dev_TO_O = nullptr;
    int capacity = 0;
    std::vector<T> edges_h, TO_E_h, TO_O_h;
    cudaEvent_t start, stop;

  public:
    T* subpix_edge_pts_final;
    T* TO_edgemap;
    T* TO_orientation;
    int edge_pt_list_idx;
    int num_of_edge_data;
    double time_nms, time_conv, time_correct;

    SubpixelTOCorrectionGPU(int H, int W, T threshold, T g_sigma, int cpu_nthreads, int n = 0)
        : img_height(H), img_width(W), interp_n(n < 0 ? 0 : n), thresh(threshold), sigma(g_sigma)
    {
        (void)cpu_nthreads;
        neighbor_radius = T(2);
        output_dir = "./output_files";
        num_of_edge_data = 4;
        edge_pt_list_idx = 0;
        time_nms = time_conv = time_correct = 0;
        const int scale = 1 << interp_n;
        work_height = (img_height - 1) * scale + 1;
        work_width = (img_width - 1) * scale + 1;
        capacity = work_height * work_width;  // the reference's subpix_edge_pts_final holds one edgel per work pixel
        const size_t px = (size_t)H * W;
        edges_h.assign((size_t)capacity * 4, T(0));
        TO_E_h.assign(px, T(0));
        TO_O_h.assign(px, T(0));
        subpix_edge_pts_final = edges_h.data();
        TO_edgemap = TO_E_h.data();
        TO_orientation = TO_O_h.data();
        int device = 0;
        toed_shim::report_cuda(cudaGetDevice(&device), "cudaGetDevice");
        toed_shim::report(toed_create(&ctx, device), "toed_create");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_E, sizeof(T) * px), "cudaMalloc");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_theta, sizeof(T) * px), "cudaMalloc");
        toed_shim::report_cuda(cudaMemset(dev_E, 0, sizeof(T) * px), "cudaMemset");
        toed_shim::report_cuda(cudaMemset(dev_theta, 0, sizeof(T) * px), "cudaMemset");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_edges, sizeof(T) * 4 * (size_t)capacity), "cudaMalloc");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_count, sizeof(int)), "cudaMalloc");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_TO_E, sizeof(T) * px), "cudaMalloc");
        toed_shim::report_cuda(cudaMalloc((void**)&dev_TO_O, sizeof(T) * px), "cudaMalloc");
        toed_shim::report_cuda(cudaEventCreate(&start), "cudaEventCreate");
        toed_shim::report_cuda(cudaEventCreate(&stop), "cudaEventCreate");
    }
    ~SubpixelTOCorrectionGPU()
    {
        cudaFree(dev_E);
        cudaFree(dev_theta);
        cudaFree(dev_edges);
        cudaFree(dev_count);
        cudaFree(dev_TO_E);
        cudaFree(dev_TO_O);
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        if (ctx) toed_destroy(ctx);
    }
    SubpixelTOCorrectionGPU(const SubpixelTOCorrectionGPU&) = delete;
    SubpixelTOCorrectionGPU& operator=(const SubpixelTOCorrectionGPU&) = delete;

    void set_edgemap(const T* data)
    {
        toed_shim::report_cuda(cudaMemcpy(dev_E, data, sizeof(T) * (size_t)img_height * img_width,
                                          cudaMemcpyHostToDevice),
                               "cudaMemcpy");
    }
    void set_orientation(const T* data)
    {
        toed_shim::report_cuda(cudaMemcpy(dev_theta, data, sizeof(T) * (size_t)img_height * img_width,
                                          cudaMemcpyHostToDevice),
                               "cudaMemcpy");
        estimate = false;
    }
    // subpix_to_correction.cpp:307-375, run on the device inside run()
    void estimate_orientation() { estimate = true; }

    // subpix_to_correction.cpp:623-736: NMS along the orientation, the eight
    // Gaussian-derivative convolutions, the per-edgel correction, isolated
    // edgels removed, dense TO_edgemap / TO_orientation; returns the count
    int run(T* edginfo_out)
    {
        toed_edgemap m;
        m.E = dev_E;
        m.theta = estimate ? nullptr : dev_theta;
        m.height = img_height;
        m.width = img_width;
        m.pitch = img_width;
        m.dtype = sizeof(T) == 8 ? TOED_F64 : TOED_F32;
        m.edgels = dev_edges;
        m.capacity = capacity;
        m.count = dev_count;
        m.TO_E = dev_TO_E;
        m.TO_O = dev_TO_O;
        toed_subpix_params p;
        p.thresh = (float)thresh;
        p.sigma = (float)sigma;
        p.nbr_radius = (float)neighbor_radius;
        p.out_dtype = sizeof(T) == 8 ? TOED_F64 : TOED_F32;
        p.precision = TOED_HYBRID;
        p.interp_n = interp_n;
        float ms = 0.f;
        toed_shim::report_cuda(cudaEventRecord(start), "cudaEventRecord");
        toed_shim::report(toed_subpix_to_correct_batch(ctx, &m, 1, &p, 0), "toed_subpix_to_correct_batch");
        toed_shim::report_cuda(cudaEventRecord(stop), "cudaEventRecord");
        toed_shim::report_cuda(cudaEventSynchronize(stop), "cudaEventSynchronize");
        toed_shim::report_cuda(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
        time_conv = ms * 1e-3;
        time_nms = 0;
        std::cout << "- Time of TO correction (GPU): " << ms << " (ms)" << std::endl;
        toed_shim::report_cuda(cudaEventRecord(start), "cudaEventRecord");
        int n = 0;
        toed_shim::report_cuda(cudaMemcpy(&n, dev_count, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        const int k = n < capacity ? n : capacity;
        std::fill(edges_h.begin(), edges_h.end(), T(0));
        if (k > 0)
            toed_shim::report_cuda(cudaMemcpy(edges_h.data(), dev_edges, sizeof(T) * 4 * (size_t)k,
                                              cudaMemcpyDeviceToHost),
                                   "cudaMemcpy");
        const size_t px = (size_t)img_height * img_width;
        toed_shim::report_cuda(cudaMemcpy(TO_E_h.data(), dev_TO_E, sizeof(T) * px, cudaMemcpyDeviceToHost),
                               "cudaMemcpy");
        toed_shim::report_cuda(cudaMemcpy(TO_O_h.data(), dev_TO_O, sizeof(T) * px, cudaMemcpyDeviceToHost),
                               "cudaMemcpy");
        toed_shim::report_cuda(cudaEventRecord(stop), "cudaEventRecord");
        toed_shim::report_cuda(cudaEventSynchronize(stop), "cudaEventSynchronize");
        toed_shim::report_cuda(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
        time_correct = ms * 1e-3;
        edge_pt_list_idx = k;
        if (edginfo_out && k > 0) std::memcpy(edginfo_out, edges_h.data(), sizeof(T) * 4 * (size_t)k);
        return k;
    }

    void set_output_dir(const std::string& dir) { output_dir = dir.empty() ? "./output_files" : dir; }
    void set_neighbor_radius(T radius) { neighbor_radius = radius; }

    // subpix_to_correction.cpp:750-776 (default stream precision, tab separated)
    void write_array_to_file(std::string filename, T* wr_data, int first_dim, int second_dim)
    {
        std::cout << "writing data to a file " << filename << " ..." << std::endl;
        if (wr_data == nullptr || first_dim <= 0 || second_dim <= 0) {
            std::cout << "write data file skipped: invalid buffer or dimensions." << std::endl;
            return;
        }
        std::string out_file_name = output_dir;
        if (!out_file_name.empty() && out_file_name.back() != '/') out_file_name.push_back('/');
        out_file_name.append(filename);
        std::ofstream out_file(out_file_name);
        if (!out_file.is_open()) {
            std::cout << "write data file cannot be opened!" << std::endl;
            return;
        }
        for (int i = 0; i < first_dim; i++) {
            for (int j = 0; j < second_dim; j++) out_file << wr_data[(size_t)i * second_dim + j] << "\t";
            out_file << "\n";
        }
    }
};
