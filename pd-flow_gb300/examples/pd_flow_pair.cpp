// Offline pair evaluator over the GB300 solver: the command line of the
// reference's Scene-Flow-Impair (main_scene_flow_impair.cpp:58-129) with
// binary PGM frames instead of PNG (no OpenCV):
//
//   pd_flow_pair [--rows r] [--i1 f] [--i2 f] [--z1 f] [--z2 f] [--out root] [--no-show]
//
//   --i1/--i2 : 8-bit PGM (P5, maxval 255) intensity images, 640x480 or 320x240
//   --z1/--z2 : 16-bit PGM (P5, maxval > 255, big-endian) depth images, metres*5000
//   --out     : results go to <root>_resultsNN.txt (lines "v u dx dy dz", row-major
//               order, scene_flow_impair.cpp:315-344) and <root>_representationNN.ppm
//               (|dx|,|dy|,|dz| scaled to 255 as blue/green/red, :280-309)
//   --no-show : accepted for compatibility (nothing is ever displayed)
//
// Build:  g++ -std=c++17 -O2 -I include -I pd-flow_gb300/csrc pd-flow_gb300/examples/pd_flow_pair.cpp \
//             -L pd-flow_gb300/lib -lpdflow_gb300 -Wl,-rpath,$PWD/pd-flow_gb300/lib -o pd_flow_pair
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "pd_flow.hpp"

namespace {

struct Args {
    unsigned rows = 240;
    std::string i1 = "i1.pgm", i2 = "i2.pgm", z1 = "z1.pgm", z2 = "z2.pgm", out = "pdflow";
    bool help = false;
};

bool parse(int argc, char** argv, Args& a)
{
    for (int i = 1; i < argc; ++i) {
        std::string k = argv[i];
        auto next = [&](std::string& dst) {
            if (i + 1 >= argc) return false;
            dst = argv[++i];
            return true;
        };
        if (k == "--help") { a.help = true; return true; }
        if (k == "--rows") {
            std::string v;
            if (!next(v)) return false;
            const int r = std::atoi(v.c_str());
            if (r != 15 && r != 30 && r != 60 && r != 120 && r != 240 && r != 480) return false;
            a.rows = unsigned(r);
        } else if (k == "--i1") { if (!next(a.i1)) return false; }
        else if (k == "--i2") { if (!next(a.i2)) return false; }
        else if (k == "--z1") { if (!next(a.z1)) return false; }
        else if (k == "--z2") { if (!next(a.z2)) return false; }
        else if (k == "--out") { if (!next(a.out)) return false; }
        else if (k == "--no-show") {}
        else return false;
    }
    return true;
}

// Reads a binary PGM; 16-bit samples are big-endian per the format.
bool read_pgm(const std::string& path, unsigned& w, unsigned& h, std::vector<uint16_t>& px, unsigned& maxval)
{
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[3] = {0};
    bool ok = std::fscanf(f, "%2s", magic) == 1 && std::strcmp(magic, "P5") == 0;
    auto read_num = [&](unsigned& v) {
        int c;
        while ((c = std::fgetc(f)) != EOF) {
            if (c == '#') { while ((c = std::fgetc(f)) != EOF && c != '\n') {} continue; }
            if (c >= '0' && c <= '9') { std::ungetc(c, f); break; }
        }
        return std::fscanf(f, "%u", &v) == 1;
    };
    ok = ok && read_num(w) && read_num(h) && read_num(maxval);
    if (ok) std::fgetc(f);
    if (ok) {
        const size_t n = size_t(w) * h;
        px.resize(n);
        if (maxval < 256) {
            std::vector<uint8_t> b(n);
            ok = std::fread(b.data(), 1, n, f) == n;
            for (size_t i = 0; ok && i < n; ++i) px[i] = b[i];
        } else {
            std::vector<uint8_t> b(2 * n);
            ok = std::fread(b.data(), 1, 2 * n, f) == 2 * n;
            for (size_t i = 0; ok && i < n; ++i) px[i] = uint16_t((b[2 * i] << 8) | b[2 * i + 1]);
        }
    }
    std::fclose(f);
    return ok;
}

bool file_exists(const std::string& p)
{
    std::FILE* f = std::fopen(p.c_str(), "rb");
    if (f) std::fclose(f);
    return f != nullptr;
}

}  // namespace

int main(int argc, char** argv)
{
    Args a;
    if (!parse(argc, argv, a) || a.help) {
        std::printf(" --rows r: 15, 30, 60, 120, 240 or 480\n --i1/--i2 <8-bit pgm>  --z1/--z2 <16-bit pgm>\n"
                    " --out <root>  --no-show\n");
        return 1;
    }
    unsigned w[4], h[4], mx[4];
    std::vector<uint16_t> img[4];
    const std::string* files[4] = {&a.i1, &a.z1, &a.i2, &a.z2};
    for (int k = 0; k < 4; ++k)
        if (!read_pgm(*files[k], w[k], h[k], img[k], mx[k])) {
            std::printf("\nThe image (%s) cannot be read\n", files[k]->c_str());
            return 1;
        }
    for (int k = 1; k < 4; ++k)
        if (w[k] != w[0] || h[k] != h[0]) {
            std::printf("image sizes differ\n");
            return 1;
        }
    try {
        pdflow::PD_flow sf(a.rows);
        sf.initializeCUDA(w[0], h[0]);
        std::vector<uint8_t> i1(img[0].begin(), img[0].end()), i2(img[2].begin(), img[2].end());
        sf.loadRGBDFrames(i1.data(), img[1].data(), i2.data(), img[3].data());
        sf.solveSceneFlowGPU();

        int nf = 0;
        char name[512];
        do {
            ++nf;
            std::snprintf(name, sizeof name, "%s_results%02d.txt", a.out.c_str(), nf);
        } while (file_exists(name));
        std::ofstream res(name);
        std::printf("Saving the estimated scene flow to file: %s \n", name);
        const unsigned R = sf.rows, C = sf.cols;
        for (unsigned v = 0; v < R; ++v)
            for (unsigned u = 0; u < C; ++u)
                res << v << " " << u << " " << sf.dxp[v + u * R] << " " << sf.dyp[v + u * R] << " "
                    << sf.dzp[v + u * R] << "\n";
        float m[3] = {0.f, 0.f, 0.f};
        const std::vector<float>* comp[3] = {&sf.dxp, &sf.dyp, &sf.dzp};
        for (int c = 0; c < 3; ++c)
            for (float x : *comp[c]) m[c] = std::fmax(m[c], std::fabs(x));
        std::snprintf(name, sizeof name, "%s_representation%02d.ppm", a.out.c_str(), nf);
        std::FILE* f = std::fopen(name, "wb");
        if (f) {
            std::fprintf(f, "P6\n%u %u\n255\n", C, R);
            for (unsigned v = 0; v < R; ++v)
                for (unsigned u = 0; u < C; ++u) {
                    // OpenCV's Vec3b is B,G,R = |dx|,|dy|,|dz|; PPM stores R,G,B.
                    uint8_t rgb[3];
                    for (int c = 0; c < 3; ++c) {
                        const float x = m[2 - c] > 0.f ? 255.f * std::fabs((*comp[2 - c])[v + u * R]) / m[2 - c] : 0.f;
                        rgb[c] = uint8_t(x);
                    }
                    std::fwrite(rgb, 1, 3, f);
                }
            std::fclose(f);
            std::printf("Saving the visual representation to file: %s \n", name);
        }
        sf.freeGPUMemory();
    } catch (const std::exception& e) {
        std::printf("%s\n", e.what());
        return 2;
    }
    return 0;
}
