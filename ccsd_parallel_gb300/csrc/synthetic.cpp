// Seeded synthetic closed-shell systems (host only).
//
// Counter-based stream: draw(key, i) = mix64(key + (i+1) * GOLDEN), with
// mix64 the SplitMix64 output function (Steele, Lea & Flood, OOPSLA 2014);
// key = mix64(seed + stream * STREAM_MUL).  Normal deviates use Box-Muller on
// draws 2i and 2i+1.  Orbital energies: occupied U[-2.0,-0.3], virtual
// U[0.1,3.0], each sorted ascending.  DF factors B[Q][p][q] =
// 0.05 z / sqrt(naux) for p <= q, mirrored to q < p.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/ccsd_gb300.h"

namespace {
constexpr uint64_t GOLDEN = 0x9E3779B97F4A7C15ull;
constexpr uint64_t STREAM_MUL = 0xD1B54A32D192ED03ull;

inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t key_of(uint64_t seed, uint64_t stream) { return mix64(seed + stream * STREAM_MUL); }
inline uint64_t draw(uint64_t key, uint64_t i) { return mix64(key + (i + 1) * GOLDEN); }
inline double uniform(uint64_t key, uint64_t i) { return (double)(draw(key, i) >> 11) * 0x1.0p-53; }
inline double normal(uint64_t key, uint64_t i) {
    double u1 = ((double)(draw(key, 2 * i) >> 11) + 1.0) * 0x1.0p-53;
    double u2 = (double)(draw(key, 2 * i + 1) >> 11) * 0x1.0p-53;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
}
}  // namespace

extern "C" int ccsd_make_synthetic(int32_t nocc, int32_t nvir, int32_t naux, uint64_t seed,
                                   double *fock, double *df) {
    if (nocc <= 0 || nvir <= 0 || naux < 0) return CCSD_ERR_INVALID_ARG;
    const int n = nocc + nvir;
    if (fock) {
        const uint64_t ko = key_of(seed, 1), kv = key_of(seed, 2);
        std::vector<double> eo(nocc), ev(nvir);
        for (int i = 0; i < nocc; ++i) eo[i] = -2.0 + (-0.3 - -2.0) * uniform(ko, i);
        for (int a = 0; a < nvir; ++a) ev[a] = 0.1 + (3.0 - 0.1) * uniform(kv, a);
        std::sort(eo.begin(), eo.end());
        std::sort(ev.begin(), ev.end());
        for (size_t k = 0; k < (size_t)n * n; ++k) fock[k] = 0.0;
        for (int i = 0; i < nocc; ++i) fock[(size_t)i * n + i] = eo[i];
        for (int a = 0; a < nvir; ++a) fock[(size_t)(nocc + a) * n + nocc + a] = ev[a];
    }
    if (df && naux > 0) {
        const uint64_t kb = key_of(seed, 3);
        const double sig = 0.05 / std::sqrt((double)naux);
        for (int q = 0; q < naux; ++q) {
            double *bq = df + (size_t)q * n * n;
            for (int p = 0; p < n; ++p)
                for (int r = p; r < n; ++r) {
                    const uint64_t idx = ((uint64_t)q * n + p) * n + r;
                    const double x = sig * normal(kb, idx);
                    bq[(size_t)p * n + r] = x;
                    bq[(size_t)r * n + p] = x;
                }
        }
    }
    return CCSD_OK;
}
