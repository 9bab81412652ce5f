// shuffle.cpp -- the reference's train shuffle for the CPU reference arm.
//
// TEST INFRASTRUCTURE ONLY.  main.cpp:303-306 shuffles the train entries with
// std::shuffle and std::mt19937(42); this calls the same two library
// templates on an index vector and permutes the caller's coordinates and
// values with it, so the oracle side reproduces the reference's order
// without the product library.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

extern "C" int orc_shuffle(int32_t* xyz, double* val, int64_t n, uint32_t seed)
{
    if (n <= 1)
        return 0;
    std::vector<int64_t> perm((size_t)n);
    for (int64_t i = 0; i < n; i++)
        perm[(size_t)i] = i;
    std::mt19937 rng(seed);
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<int32_t> nx((size_t)n * 3);
    std::vector<double> nv((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const int64_t s = perm[(size_t)i];
        std::memcpy(&nx[(size_t)(3 * i)], xyz + 3 * s, 12);
        nv[(size_t)i] = val[s];
    }
    std::memcpy(xyz, nx.data(), sizeof(int32_t) * 3 * (size_t)n);
    std::memcpy(val, nv.data(), sizeof(double) * (size_t)n);
    return 0;
}
