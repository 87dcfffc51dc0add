// toed_batch -- the batch driver that replaces the reference's
// run_gpu_batch.sh (one TOED process per image, run_gpu_batch.sh:1-24) and
// its per-image decode (main_gpu_cpu.cpp:101-131): every image of a folder
// is decoded on host threads into page-locked buffers, up to 64 images go to
// the GPU in one toed_detect_host_batch call while the next group is being
// decoded, and each image's edgel list is written as
// <output_dir>/<image basename>_edges_gpu.txt in the reference's GPU file
// format (data_final_output_gpu.txt: 10 significant digits, a tab after
// every value, gpu_toed.hpp:452-478).
//
//   toed_batch <input_dir> <output_dir> [-g GPU] [-e EXT,EXT...] [-s SIGMA]
//              [--float-output] [--qad]
//
// Decoding: binary (P5) and plain (P2) PGM, 8 or 16 bits per sample; samples
// of a maximum value other than 255 are scaled to 0..255 (rounded).  Other
// formats need a decoder that is not part of this build and are skipped with
// a message.  The reference's no-OpenCV path reads the
// header's final whitespace byte as pixel (0, 0); this driver decodes the
// raster the way its OpenCV path does.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include <dirent.h>
#include <cuda_runtime.h>

#include "../../include/toed_gb300.h"

namespace {

struct Image {
    std::string name;        // basename without extension
    int H = 0, W = 0;
    unsigned char* px = nullptr;  // page-locked, H x W
    std::string error;
};

bool ends_with_ci(const std::string& s, const std::string& ext)
{
    if (s.size() <= ext.size() + 1 || s[s.size() - ext.size() - 1] != '.') return false;
    for (size_t i = 0; i < ext.size(); ++i)
        if (std::tolower((unsigned char)s[s.size() - ext.size() + i]) != std::tolower((unsigned char)ext[i]))
            return false;
    return true;
}

// next header token of a PGM file, skipping whitespace and '#' comments
bool pgm_token(std::istream& in, std::string& tok)
{
    tok.clear();
    int c;
    while ((c = in.get()) != EOF) {
        if (c == '#') {
            while ((c = in.get()) != EOF && c != '\n' && c != '\r') {
            }
            continue;
        }
        if (!std::isspace(c)) break;
    }
    if (c == EOF) return false;
    do {
        tok.push_back((char)c);
    } while ((c = in.get()) != EOF && !std::isspace(c) && c != '#');
    if (c == '#') in.unget();
    return true;  // the whitespace byte after the token has been consumed
}

void decode_pgm(const std::string& path, Image& im)
{
    std::ifstream in(path, std::ios::binary);
    std::string magic, ws, hs, ms;
    if (!in || !pgm_token(in, magic) || (magic != "P5" && magic != "P2") || !pgm_token(in, ws) ||
        !pgm_token(in, hs) || !pgm_token(in, ms)) {
        im.error = "not a PGM image";
        return;
    }
    const long W = std::strtol(ws.c_str(), nullptr, 10), H = std::strtol(hs.c_str(), nullptr, 10);
    const long maxv = std::strtol(ms.c_str(), nullptr, 10);
    if (W <= 0 || H <= 0 || W > 65535 || H > 65535 || maxv <= 0 || maxv > 65535) {
        im.error = "bad PGM header";
        return;
    }
    im.H = (int)H;
    im.W = (int)W;
    if (cudaHostAlloc((void**)&im.px, (size_t)H * W, cudaHostAllocDefault) != cudaSuccess) {
        im.error = "cudaHostAlloc failed";
        im.px = nullptr;
        return;
    }
    const size_t n = (size_t)H * W;
    auto to8 = [&](long v) -> unsigned char {
        if (maxv == 255) return (unsigned char)std::min(v, 255L);
        return (unsigned char)std::min(255L, (v * 255 + maxv / 2) / maxv);
    };
    if (magic == "P5") {
        const int bps = maxv < 256 ? 1 : 2;
        std::vector<unsigned char> raw(n * bps);
        in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)raw.size());
        if ((size_t)in.gcount() != raw.size()) {
            im.error = "truncated PGM raster";
            return;
        }
        for (size_t k = 0; k < n; ++k)
            im.px[k] = bps == 1 ? to8(raw[k]) : to8(((long)raw[2 * k] << 8) | raw[2 * k + 1]);
    } else {
        for (size_t k = 0; k < n; ++k) {
            long v;
            if (!(in >> v)) {
                im.error = "truncated PGM raster";
                return;
            }
            im.px[k] = to8(v);
        }
    }
}

}  // namespace

static int usage(const char* argv0)
{
    std::cout << "Usage: " << argv0 << " <input_dir> <output_dir> [-g GPU] [-e EXT,EXT...] [-s SIGMA]\n"
              << "       [--float-output] [--qad]\n"
              << "Writes <output_dir>/<image basename>_edges_gpu.txt for every image (PGM) of input_dir.\n";
    return 0;
}

static bool mkdir_p(const std::string& dir)
{
    std::string cur;
    std::stringstream ss(dir);
    std::string part;
    if (!dir.empty() && dir[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
    }
    return true;
}

int main(int argc, char** argv)
{
    std::string in_dir, out_dir, exts = "pgm";
    int gpu = 0, out_dtype = TOED_F64, orientation = TOED_ORI_GRID;
    float sigma = 2.0f;  // the reference's fixed sigma and kernel (main_gpu_cpu.cpp:154-155)
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if ((a == "-g" || a == "--gpu-id") && i + 1 < argc) gpu = std::atoi(argv[++i]);
        else if ((a == "-e" || a == "--ext") && i + 1 < argc) exts = argv[++i];
        else if ((a == "-s" || a == "--sigma") && i + 1 < argc) sigma = (float)std::atof(argv[++i]);
        else if (a == "--float-output") out_dtype = TOED_F32;
        else if (a == "--qad") orientation = TOED_ORI_QAD;
        else if (a == "-h" || a == "--help") return usage(argv[0]);
        else if (!a.empty() && a[0] == '-') { std::cerr << "Unknown option: " << a << "\n"; return 1; }
        else if (in_dir.empty()) in_dir = a;
        else if (out_dir.empty()) out_dir = a;
        else { std::cerr << "Unexpected argument: " << a << "\n"; return 1; }
    }
    if (in_dir.empty() || out_dir.empty()) return usage(argv[0]), 1;
    std::vector<std::string> ext_list;
    {
        std::stringstream ss(exts);
        std::string e;
        while (std::getline(ss, e, ',')) if (!e.empty()) ext_list.push_back(e);
    }
    std::vector<std::string> files;
    if (DIR* d = opendir(in_dir.c_str())) {
        while (dirent* e = readdir(d)) {
            const std::string f = e->d_name;
            for (const auto& x : ext_list)
                if (ends_with_ci(f, x)) { files.push_back(f); break; }
        }
        closedir(d);
    } else {
        std::cerr << "Input directory not found: " << in_dir << "\n";
        return 1;
    }
    std::sort(files.begin(), files.end());
    if (!mkdir_p(out_dir)) { std::cerr << "Cannot create " << out_dir << "\n"; return 1; }
    if (cudaSetDevice(gpu) != cudaSuccess) { std::cerr << "cudaSetDevice failed\n"; return 1; }
    toed_ctx* ctx = nullptr;
    if (toed_create(&ctx, gpu) != TOED_OK) { std::cerr << "toed_create failed\n"; return 1; }
    toed_params prm;
    toed_params_default(&prm, sigma);
    prm.out_dtype = out_dtype;
    prm.orientation = orientation;
    const int rec = out_dtype == TOED_F64 ? 32 : 16;

    // groups of up to 64 images: the next group is decoded on a host thread
    // while the current one is detected and written
    const size_t G = 64;
    auto decode_group = [&](size_t b, std::vector<Image>& grp) {
        grp.clear();
        for (size_t i = b; i < std::min(files.size(), b + G); ++i) {
            Image im;
            im.name = files[i].substr(0, files[i].rfind('.'));
            decode_pgm(in_dir + "/" + files[i], im);
            grp.push_back(im);
        }
    };
    unsigned char* out_arena = nullptr;  // page-locked edgel lists of a group
    size_t out_cap = 0;
    int* counts = nullptr;
    cudaHostAlloc((void**)&counts, sizeof(int) * G, cudaHostAllocDefault);
    int written = 0, failed = 0;
    std::vector<Image> cur, next;
    decode_group(0, cur);
    for (size_t b = 0; b < files.size(); b += G) {
        std::thread th;
        if (b + G < files.size()) th = std::thread(decode_group, b + G, std::ref(next));
        std::vector<toed_host_image> arr;
        std::vector<size_t> slot;  // index into cur of each detected image
        size_t need = 0;
        for (size_t i = 0; i < cur.size(); ++i) {
            if (!cur[i].error.empty()) {
                std::cerr << cur[i].name << ": " << cur[i].error << " (skipped)\n";
                ++failed;
                continue;
            }
            need += (size_t)cur[i].H * cur[i].W * rec;  // capacity H x W edgels (one per pixel)
        }
        if (need > out_cap) {
            if (out_arena) cudaFreeHost(out_arena);
            out_arena = nullptr;
            out_cap = 0;
            if (cudaHostAlloc((void**)&out_arena, need, cudaHostAllocDefault) == cudaSuccess) out_cap = need;
        }
        size_t off = 0;
        for (size_t i = 0; i < cur.size() && out_cap >= need; ++i) {
            if (!cur[i].error.empty()) continue;
            toed_host_image h;
            h.pixels = cur[i].px;
            h.height = cur[i].H;
            h.width = cur[i].W;
            h.pitch = cur[i].W;
            h.dtype = TOED_U8;
            h.edgels = out_arena + off;
            h.capacity = cur[i].H * cur[i].W;
            h.count = counts + arr.size();
            h.grid_index = nullptr;
            off += (size_t)h.capacity * rec;
            arr.push_back(h);
            slot.push_back(i);
        }
        toed_status st = arr.empty() ? TOED_OK : toed_detect_host_batch(ctx, arr.data(), (int)arr.size(), &prm, (int)arr.size(), 0);  // one image per copy group
        if (out_cap < need) st = TOED_ERR_CAPACITY;
        for (size_t k = 0; k < arr.size(); ++k) {
            Image& im = cur[slot[k]];
            const std::string path = out_dir + "/" + im.name + "_edges_gpu.txt";
            std::vector<unsigned char> big;  // an image with more edgels than pixels: again with room for all
            const void* edg = arr[k].edgels;
            int n = counts[k];
            toed_status sti = st;
            if (sti == TOED_OK && n > arr[k].capacity) {
                big.resize((size_t)4 * im.H * im.W * rec);
                toed_host_image h = arr[k];
                h.edgels = big.data();
                h.capacity = 4 * im.H * im.W;
                sti = toed_detect_host_batch(ctx, &h, 1, &prm, 1, 0);
                n = *h.count;
                edg = big.data();
            }
            if (sti == TOED_OK) sti = toed_write_edgels_txt(path.c_str(), edg, out_dtype, n, 10);
            if (sti != TOED_OK) {
                std::cerr << im.name << ": " << toed_status_string(sti) << "\n";
                ++failed;
            } else {
                ++written;
            }
        }
        for (auto& im : cur)
            if (im.px) cudaFreeHost(im.px);
        if (th.joinable()) th.join();
        std::swap(cur, next);
    }
    if (out_arena) cudaFreeHost(out_arena);
    cudaFreeHost(counts);
    toed_destroy(ctx);
    std::cout << "toed_batch: " << written << " edge lists written to " << out_dir << ", " << failed << " failed\n";
    return failed ? 1 : 0;
}
