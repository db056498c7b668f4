// Shared pieces of the drop-in `uniform` and `amr` programs: flag parsing and the VTK writers.
//
// Flags follow the reference's parsing rule: a flag is honoured only when a value follows it
// (src/tgv3d_uniform.cu:92-94, src/tgv3d_amr.cu:565-567), so `--bench` alone is ignored and
// `--bench 1` enables it.  The .vti/.vtp files are byte-compatible with the reference's writers
// (src/tgv3d_uniform.cu:110-140, src/tgv3d_amr.cu:602-641) because the readers of
// scripts/preview_tgv3d.py:21-42 depend on that layout: XML header, "_" then per array a UInt64 byte
// count and the raw little-endian Float32 payload.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "jp.h"

namespace cli {

inline const char* find(int c, char** v, const char* k) {
    for (int i = 1; i < c - 1; ++i)
        if (!std::strcmp(v[i], k)) return v[i + 1];
    return nullptr;
}
inline int argi(int c, char** v, const char* k, int d) {
    const char* s = find(c, v, k);
    return s ? std::atoi(s) : d;
}
inline double argd(int c, char** v, const char* k, double d) {
    const char* s = find(c, v, k);
    return s ? std::atof(s) : d;
}
inline const char* args(int c, char** v, const char* k, const char* d) {
    const char* s = find(c, v, k);
    return s ? s : d;
}

inline int storage_of(const char* p) {
    if (!std::strcmp(p, "fp16")) return JP_FP16;
    if (!std::strcmp(p, "bf16")) return JP_BF16;
    if (!std::strcmp(p, "fp64")) return JP_FP64;
    return JP_FP32;
}
inline int refine_of(const char* m) {
    if (!std::strcmp(m, "all")) return JP_REFINE_ALL;
    if (!std::strcmp(m, "slab")) return JP_REFINE_SLAB;
    return JP_REFINE_SENSOR;
}

// one appended raw array: UInt64 byte count, then the bytes
inline void put_array(FILE* f, const std::vector<float>& a) {
    uint64_t nb = uint64_t(a.size()) * 4;
    std::fwrite(&nb, 8, 1, f);
    std::fwrite(a.data(), 1, nb, f);
}

// ImageData with Q, speed and (when vel is non-empty) the velocity vector
inline bool write_vti(const std::string& path, const std::vector<float>& Q, const std::vector<float>& spd,
                      const std::vector<float>& vel, int N) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "open %s\n", path.c_str());
        return false;
    }
    const bool withVel = !vel.empty();
    const uint64_t nb1 = uint64_t(Q.size()) * 4, nb2 = uint64_t(spd.size()) * 4;
    const uint64_t o0 = 0, o1 = 8 + nb1, o2 = o1 + 8 + nb2;
    std::fprintf(f, "<?xml version=\"1.0\"?>\n");
    std::fprintf(f, "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
    std::fprintf(f, "  <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n", N - 1, N - 1, N - 1);
    std::fprintf(f, "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n", N - 1, N - 1, N - 1);
    if (withVel) std::fprintf(f, "      <PointData Scalars=\"Q\" Vectors=\"velocity\">\n");
    else std::fprintf(f, "      <PointData Scalars=\"Q\">\n");
    std::fprintf(f, "        <DataArray type=\"Float32\" Name=\"Q\" format=\"appended\" offset=\"%llu\"/>\n", (unsigned long long)o0);
    std::fprintf(f, "        <DataArray type=\"Float32\" Name=\"speed\" format=\"appended\" offset=\"%llu\"/>\n", (unsigned long long)o1);
    if (withVel)
        std::fprintf(f, "        <DataArray type=\"Float32\" Name=\"velocity\" NumberOfComponents=\"3\" format=\"appended\" offset=\"%llu\"/>\n",
                     (unsigned long long)o2);
    std::fprintf(f, "      </PointData>\n    </Piece>\n  </ImageData>\n");
    std::fprintf(f, "  <AppendedData encoding=\"raw\">\n_");
    put_array(f, Q);
    put_array(f, spd);
    if (withVel) put_array(f, vel);
    std::fprintf(f, "\n  </AppendedData>\n</VTKFile>\n");
    std::fclose(f);
    return true;
}

struct Box {
    double x0, y0, z0, s;
    int lv;
};

// PolyData of wire-frame boxes (8 points, 12 lines each) with an Int32 point field "level"
inline bool write_boxes(const std::string& path, const std::vector<Box>& bs) {
    const int nb = (int)bs.size();
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "<?xml version=\"1.0\"?>\n<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\">\n  <PolyData>\n");
    std::fprintf(f, "    <Piece NumberOfPoints=\"%d\" NumberOfLines=\"%d\">\n", nb * 8, nb * 12);
    std::fprintf(f, "      <PointData><DataArray type=\"Int32\" Name=\"level\" format=\"ascii\">\n");
    for (const Box& b : bs)
        for (int v = 0; v < 8; ++v) std::fprintf(f, "%d\n", b.lv);
    std::fprintf(f, "      </DataArray></PointData>\n      <Points>\n        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (const Box& b : bs) {
        const double x0 = b.x0, y0 = b.y0, z0 = b.z0, s = b.s;
        const double cx[8] = {x0, x0 + s, x0, x0 + s, x0, x0 + s, x0, x0 + s};
        const double cy[8] = {y0, y0, y0 + s, y0 + s, y0, y0, y0 + s, y0 + s};
        const double cz[8] = {z0, z0, z0, z0, z0 + s, z0 + s, z0 + s, z0 + s};
        for (int v = 0; v < 8; ++v) std::fprintf(f, "%g %g %g\n", cx[v], cy[v], cz[v]);
    }
    std::fprintf(f, "        </DataArray>\n      </Points>\n      <Lines>\n        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n");
    static const int E12[12][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3}, {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    for (int bi = 0; bi < nb; ++bi)
        for (int e = 0; e < 12; ++e) std::fprintf(f, "%d %d\n", bi * 8 + E12[e][0], bi * 8 + E12[e][1]);
    std::fprintf(f, "        </DataArray>\n        <DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n");
    for (int e = 0; e < nb * 12; ++e) std::fprintf(f, "%d\n", (e + 1) * 2);
    std::fprintf(f, "        </DataArray>\n      </Lines>\n    </Piece>\n  </PolyData>\n</VTKFile>\n");
    std::fclose(f);
    return true;
}

// C ABI call or exit 2 (the reference's CK() exit code, src/tgv3d_uniform.cu:25-26)
inline void ck(jp_status st, const char* what) {
    if (st != JP_OK) {
        std::fprintf(stderr, "jp %s: %s\n", what, jp_last_error());
        std::exit(2);
    }
}

}  // namespace cli
