/* bm_oracle_params.cpp -- the oracle's BRIEF sampling pattern (TEST INFRASTRUCTURE).
 *
 * Restates briefmatch.cpp:124-148 for the oracle, so that the CPU side of the
 * tests and the bench's reference arm can build the same pattern as the engine
 * without loading the engine library: 4N values sign(g)*g^2 with g ~ N(0, 0.2),
 * clamped to [-1, 1] and scaled by the patch radius.  The reference draws g from
 * Boost's mt19937 seeded by time(NULL); here the seed is explicit and the draws come
 * from the C++ standard library's std::mt19937_64 and std::normal_distribution<double>,
 * the generator the engine's bm_make_pattern uses, so equal seeds give equal patterns.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>

extern "C" int bmo_make_pattern(int N, float patchArea, uint64_t seed, float* out)
{
    if (N < 1 || N > 512 || !out) return -1;
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 0.2);  // briefmatch.cpp:126
    for (int s = 0; s < 4 * N; s++) {
        float val = (float)nd(rng);
        val = (2 * float(val > 0) - 1) * std::pow(std::fabs(val), 2.0f);  // briefmatch.cpp:141-143
        out[s] = patchArea * std::max(-1.0f, std::min(1.0f, val));
    }
    return 0;
}
