// subpix_driver.cpp -- a driver in the style of the reference's
// main_subpix_to_correction.cpp (:279-293) using SubpixelTOCorrectionGPU<T>
// from the header-only drop-in toed_gb300.hpp.  Built and run by
// tests/test_gpu_cpp_shim.py.
//
//   subpix_driver <raw f64 map> <H> <W> <out dir> [<raw f64 orientation>]
// writes <out dir>/sp_edges.bin (N x 4 doubles), sp_TO_E.bin, sp_TO_O.bin
// (H x W doubles; orientation estimated) and, given an orientation file,
// sp_edges_f32.bin (the float class with set_orientation).
#include <cstdio>
#include <fstream>
#include <vector>

#include "toed_gb300.hpp"

static std::vector<double> read_raw(const char* path, size_t n)
{
    std::vector<double> v(n);
    std::FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(double), n, f) != n) v.clear();
    if (f) std::fclose(f);
    return v;
}

template <typename T>
static void dump(const std::string& path, const T* p, size_t n)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    std::fwrite(p, sizeof(T), n, f);
    std::fclose(f);
}

int main(int argc, char** argv)
{
    if (argc < 5) return 2;
    const int H = std::atoi(argv[2]), W = std::atoi(argv[3]);
    const std::string out = argv[4];
    const std::vector<double> E = read_raw(argv[1], (size_t)H * W);
    if (E.empty()) return 3;
    {
        SubpixelTOCorrectionGPU<double> tc(H, W, 0.1, 2.0, 8);
        tc.set_output_dir(out);
        tc.set_edgemap(E.data());
        tc.estimate_orientation();
        tc.set_neighbor_radius(2.0);
        std::vector<double> edges((size_t)H * W * 4, 0.0);
        const int n = tc.run(edges.data());
        if (n != tc.edge_pt_list_idx) return 4;
        dump(out + "/sp_edges.bin", edges.data(), (size_t)4 * n);
        dump(out + "/sp_TO_E.bin", tc.TO_edgemap, (size_t)H * W);
        dump(out + "/sp_TO_O.bin", tc.TO_orientation, (size_t)H * W);
        tc.write_array_to_file("subpix_edges.txt", tc.subpix_edge_pts_final, n, tc.num_of_edge_data);
    }
    if (argc > 5) {
        const std::vector<double> th = read_raw(argv[5], (size_t)H * W);
        if (th.empty()) return 5;
        std::vector<float> Ef(E.begin(), E.end()), thf(th.begin(), th.end());
        SubpixelTOCorrectionGPU<float> tc(H, W, 0.1f, 2.0f, 8);
        tc.set_edgemap(Ef.data());
        tc.set_orientation(thf.data());
        std::vector<float> edges((size_t)H * W * 4, 0.f);
        const int n = tc.run(edges.data());
        dump(out + "/sp_edges_f32.bin", edges.data(), (size_t)4 * n);
    }
    return 0;
}
