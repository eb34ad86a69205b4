// Test harness (no GPU needed): the C++ drop-in class of include/ncvis.hpp
// compiles with the reference's call shapes (src/main.cpp:310-312,
// wrapper/cncvis.pxd:10-11) and reports the reference's argument errors
// (src/ncvis.cpp:364-369) as std::runtime_error before any device work.
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "ncvis.hpp"

static int expect_throw(ncvis::NCVis &vis, const float *X, size_t N, size_t D, float *Y,
                        const char *needle) {
    try {
        vis.fit_transform(X, N, D, Y);
    } catch (const std::runtime_error &e) {
        if (std::strstr(e.what(), needle)) return 0;
        std::printf("unexpected message: %s\n", e.what());
        return 1;
    }
    std::printf("no exception for: %s\n", needle);
    return 1;
}

int main() {
    size_t plan[4] = {1, 2, 3, 4};
    ncvis::NCVis vis(2, 4, 15, 16, 200, 42, 4, 20, 0.76687364f, 1.22256382f, 1.f, 1.f, plan,
                     ncvis::Distance::cosine_similarity);
    ncvis::NCVis defaults;  // the reference's C++ defaults
    float X[6] = {0, 1, 2, 3, 4, 5};
    float Y[4];
    int bad = 0;
    bad += expect_throw(vis, X, 0, 3, Y, "Dataset should have at least one element.");
    bad += expect_throw(vis, X, 2, 0, Y, "Dataset should have at least one element.");
    bad += expect_throw(vis, X, 2, 3, nullptr, "Null pointer provided for output.");
    ncvis::NCVis odd(2, 1, 15, 16, 200, 42, 50, 20, 1.f, 1.f, 1.f, 1.f, nullptr,
                     (ncvis::Distance)7);
    bad += expect_throw(odd, X, 2, 3, Y, "Unrecognized distance type.");
    if (bad) return 1;
    std::printf("ok\n");
    return 0;
}
