// shim_driver.cpp -- a reference-style driver (main_gpu_cpu.cpp:101-339) that
// uses the header-only drop-in toed_gb300.hpp exactly as the reference's own
// class and free functions are used.  Built and run by tests/test_gpu_cpp_shim.py.
//
//   shim_driver <raw u8 file> <H> <W> <out dir>
// writes <out dir>/edges_f64.bin (N x 4 doubles from ThirdOrderEdgeDetectionGPU<double>),
// <out dir>/edges_f32.bin (float variant) and <out dir>/posx.bin (gpu_convolve + gpu_nms
// position map, FP64).
#include <cstdio>
#include <fstream>
#include <vector>

#include "toed_gb300.hpp"

int main(int argc, char** argv)
{
    if (argc < 5) return 2;
    const int H = std::atoi(argv[2]), W = std::atoi(argv[3]);
    const std::string out = argv[4];
    int n64 = 0, n32 = 0;
    {
        std::ifstream in(argv[1], std::ios::binary);
        ThirdOrderEdgeDetectionGPU<double> det(0, H, W, 17, 2);
        det.set_output_dir(out);
        det.preprocessing(in);
        det.convolve_img();
        std::vector<double> edges((size_t)(2 * H) * (2 * W) * 4, 0.0);
        n64 = det.non_maximum_suppresion(edges.data());
        std::FILE* f = std::fopen((out + "/edges_f64.bin").c_str(), "wb");
        std::fwrite(edges.data(), sizeof(double), (size_t)4 * n64, f);
        std::fclose(f);
    }
    {
        std::ifstream in(argv[1], std::ios::binary);
        ThirdOrderEdgeDetectionGPU<float> det(0, H, W, 17, 2);
        det.set_output_dir(out);
        det.preprocessing(in);
        det.convolve_img();
        std::vector<float> edges((size_t)(2 * H) * (2 * W) * 4, 0.f);
        n32 = det.non_maximum_suppresion(edges.data());
        std::FILE* f = std::fopen((out + "/edges_f32.bin").c_str(), "wb");
        std::fwrite(edges.data(), sizeof(float), (size_t)4 * n32, f);
        std::fclose(f);
    }
    {
        // the reference's free-function form with its own tap arrays
        std::ifstream in(argv[1], std::ios::binary);
        std::vector<double> img((size_t)H * W);
        for (auto& v : img) v = (double)(int)in.get();
        const int H2 = 2 * H, W2 = 2 * W, n = 19;
        const double s = 2.0, nrm = std::sqrt(2.0 * 3.14159265358979323846);
        std::vector<double> taps(8 * n);
        for (int sh = 0; sh < 2; ++sh)
            for (int k = 0; k < n; ++k) {
                const double x = (double)(k - 9) + (sh ? 0.5 : 0.0), e = std::exp(-(x * x) / (2 * s * s));
                taps[(4 * sh + 0) * n + k] = e / (nrm * s);
                taps[(4 * sh + 1) * n + k] = (-x * e) / (nrm * s * s * s);
                taps[(4 * sh + 2) * n + k] = ((x * x - s * s) * e) / (nrm * s * s * s * s * s);
                taps[(4 * sh + 3) * n + k] = ((x * (3 * s * s - x * x)) * e) / (nrm * s * s * s * s * s * s * s);
            }
        double *d_img, *d_pl[4], *d_t[8], *d_px, *d_py;
        cudaMalloc(&d_img, sizeof(double) * img.size());
        cudaMemcpy(d_img, img.data(), sizeof(double) * img.size(), cudaMemcpyHostToDevice);
        for (auto& p : d_pl) cudaMalloc(&p, sizeof(double) * H2 * W2);
        for (int f = 0; f < 8; ++f) {
            cudaMalloc(&d_t[f], sizeof(double) * n);
            cudaMemcpy(d_t[f], taps.data() + f * n, sizeof(double) * n, cudaMemcpyHostToDevice);
        }
        cudaMalloc(&d_px, sizeof(double) * H2 * W2);
        cudaMalloc(&d_py, sizeof(double) * H2 * W2);
        // argument order of gpu_kernels.hpp:36-45: Gx, Gxx, Gxxx, G_of_x, Gx_sh, Gxx_sh, Gxxx_sh, G_of_x_sh
        gpu_convolve(0, H, W, H2, W2, d_img, d_pl[0], d_pl[1], d_pl[2], d_pl[3], d_t[1], d_t[2], d_t[3], d_t[0],
                     d_t[5], d_t[6], d_t[7], d_t[4]);
        gpu_nms(0, H2, W2, d_pl[0], d_pl[1], d_pl[2], d_px, d_py);
        std::vector<double> px((size_t)H2 * W2);
        cudaMemcpy(px.data(), d_px, sizeof(double) * px.size(), cudaMemcpyDeviceToHost);
        std::FILE* f = std::fopen((out + "/posx.bin").c_str(), "wb");
        std::fwrite(px.data(), sizeof(double), px.size(), f);
        std::fclose(f);
    }
    std::printf("edges %d %d\n", n64, n32);
    return 0;
}
