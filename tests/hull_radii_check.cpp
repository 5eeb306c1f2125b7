// Test helper: runs the host-side convex-mesh preparation (prepare_hull) on meshes read from a
// binary file and prints, per mesh and precision, the certified inner and outer radii followed by
// the prepared (centroid-relocated) vertices, for tests/test_hull_radii.py.
//
// Input: int H, then per mesh: int nv, int nf, int ni, double verts[nv*3], int face_off[nf+1],
// int face_idx[ni].  Output per mesh and precision (32, then 64), one line each:
// "<bits> <inner> <outer> <nv> x0 y0 z0 x1 ...".
#include <cstdio>
#include <vector>
#include "pe_host.h"

template <class R> static void emit(int bits, const pe::HullPrep<R>& h) {
    std::printf("%d %.17g %.17g %d", bits, double(h.inner), double(h.outer), (int)(h.v.size() / 3));
    for (R x : h.v) std::printf(" %.17g", double(x));
    std::printf("\n");
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int H = 0;
    if (std::fread(&H, 4, 1, f) != 1) return 2;
    for (int m = 0; m < H; m++) {
        int nv, nf, ni;
        if (std::fread(&nv, 4, 1, f) != 1 || std::fread(&nf, 4, 1, f) != 1 || std::fread(&ni, 4, 1, f) != 1) return 2;
        std::vector<double> v((size_t)nv * 3);
        std::vector<int> off(nf + 1), idx(ni);
        if (std::fread(v.data(), 8, v.size(), f) != v.size() || std::fread(off.data(), 4, off.size(), f) != off.size() ||
            std::fread(idx.data(), 4, idx.size(), f) != idx.size())
            return 2;
        emit(32, pe::prepare_hull<float>(v.data(), nv, off.data(), idx.data(), nf, false));
        emit(64, pe::prepare_hull<double>(v.data(), nv, off.data(), idx.data(), nf, false));
    }
    return 0;
}
