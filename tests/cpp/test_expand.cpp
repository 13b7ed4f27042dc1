// Host-only check of MinvExpander (csrc/frg_expand.h), the threads that expand
// packed Minv for the pipelined host-buffer call: jobs of many sizes, started
// back to back with wait() between them as that call does, must each write
// exactly the dense symmetric matrices of their own packed input and nothing
// else.  Built and run by tests/test_expand.py for several joint counts.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "frg_expand.h"

int main() {
    constexpr int N = frg::kN, P = frg::kMinvPackedN, D = frg::kMinvN;
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    int bad = 0;
    for (int threads : {1, 3, 14}) {
        MinvExpander ex(threads);
        const size_t sizes[] = {0, 1, 5, 1023, 1024, 1025, 4097, 66809, 3, 20000};
        std::vector<std::vector<float>> packed, dense;
        for (size_t n : sizes) {
            packed.emplace_back(P * n);
            for (float &x : packed.back()) x = u(rng);
            dense.emplace_back(D * n + 16, -7.0f);  // 16 guard floats past the end
        }
        for (size_t j = 0; j < sizeof(sizes) / sizeof(sizes[0]); j++) {
            ex.wait();
            ex.start(packed[j].data(), dense[j].data(), sizes[j]);
        }
        ex.wait();
        for (size_t j = 0; j < sizeof(sizes) / sizeof(sizes[0]); j++) {
            const size_t n = sizes[j];
            for (size_t k = 0; k < n; k++)
                for (int c = 0; c < N; c++)
                    for (int r = 0; r < N; r++) {
                        const int lo = r < c ? r : c, hi = r < c ? c : r;
                        const float want = packed[j][P * k + hi * (hi + 1) / 2 + lo];
                        if (dense[j][D * k + r + N * c] != want) bad++;
                    }
            for (size_t e = D * n; e < dense[j].size(); e++)
                if (dense[j][e] != -7.0f) bad++;
        }
    }
    std::printf("%s: N=%d, %d mismatches\n", bad ? "FAIL" : "OK", N, bad);
    return bad ? 1 : 0;
}
