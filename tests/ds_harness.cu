// ds_harness.cu -- host check of the double-single unit-vector updates of common.cuh:
// ds_add_renorm (updates that keep |e| = 1 to FP32 rounding: a rotation formed in FP32)
// and ds_add_renorm_wide (updates that leave the sphere at first order: an explicit
// Euler step of up to 0.2 in angle).  Random unit vectors are split into hi + lo FP32
// pairs, updated, and compared in long double with the exactly normalised sum
// hi + lo + d.  Prints one line per case: "<case> <max |norm^2 - 1|> <max component
// error> <max |lo| / ulp(hi)>"; the third case, the second-order form on first-order
// updates, shows why those take the wide form.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "../uppasd_gb300/csrc/common.cuh"

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;

double urand() {  // xorshift64*, (0, 1)
    g_state ^= g_state >> 12;
    g_state ^= g_state << 25;
    g_state ^= g_state >> 27;
    return ((double)((g_state * 2685821657736338717ull) >> 11) + 0.5) * 0x1.0p-53;
}

double nrand() {
    return std::sqrt(-2.0 * std::log(urand())) * std::cos(6.283185307179586 * urand());
}

void unit(long double v[3]) {
    long double n = 0;
    for (int c = 0; c < 3; ++c) {
        v[c] = nrand();
        n += v[c] * v[c];
    }
    n = std::sqrt(n);
    for (int c = 0; c < 3; ++c) v[c] /= n;
}

}  // namespace

int main(int argc, char **argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 100000;
    for (int kind = 0; kind < 3; ++kind) {
        const bool wide = kind >= 1;  // first-order updates
        long double max_norm = 0, max_err = 0, max_lo = 0;
        for (int t = 0; t < n; ++t) {
            long double v[3], a[3], b[3];
            unit(v);
            unit(a);
            float hi[3], lo[3], d[3];
            for (int c = 0; c < 3; ++c) {
                hi[c] = (float)v[c];
                lo[c] = (float)(v[c] - hi[c]);
            }
            const long double h = 0.2L * urand();
            // b = a x v: the tangent direction of a rotation about a
            b[0] = a[1] * v[2] - a[2] * v[1];
            b[1] = a[2] * v[0] - a[0] * v[2];
            b[2] = a[0] * v[1] - a[1] * v[0];
            if (!wide) {
                // Rodrigues rotation of the FP32 vector hi by angle h about a, formed in
                // FP32 as the kernels do; d is its change
                const float ca = (float)std::cos(h), sa = (float)std::sin(h);
                const float ax[3] = {(float)a[0], (float)a[1], (float)a[2]};
                const float ad = ax[0] * hi[0] + ax[1] * hi[1] + ax[2] * hi[2];
                const float cr[3] = {ax[1] * hi[2] - ax[2] * hi[1], ax[2] * hi[0] - ax[0] * hi[2],
                                     ax[0] * hi[1] - ax[1] * hi[0]};
                for (int c = 0; c < 3; ++c) {
                    const float r = hi[c] * ca + cr[c] * sa + ax[c] * ad * (1.0f - ca);
                    d[c] = r - hi[c];
                }
            } else {
                for (int c = 0; c < 3; ++c) d[c] = (float)(h * b[c]);
            }
            long double want[3], nw = 0;
            for (int c = 0; c < 3; ++c) {
                want[c] = (long double)hi[c] + (long double)lo[c] + (long double)d[c];
                nw += want[c] * want[c];
            }
            nw = std::sqrt(nw);
            if (kind == 1)
                uppasd::ds_add_renorm_wide(hi, lo, d);
            else
                uppasd::ds_add_renorm(hi, lo, d);
            long double n2 = 0;
            for (int c = 0; c < 3; ++c) {
                const long double e = (long double)hi[c] + (long double)lo[c];
                n2 += e * e;
                const long double err = std::fabs(e - want[c] / nw);
                if (err > max_err) max_err = err;
                const float ulp = std::nextafter(std::fabs(hi[c]), INFINITY) - std::fabs(hi[c]);
                if (hi[c] != 0.0f && std::fabs((long double)lo[c]) / ulp > max_lo)
                    max_lo = std::fabs((long double)lo[c]) / ulp;
            }
            if (std::fabs(n2 - 1) > max_norm) max_norm = std::fabs(n2 - 1);
        }
        static const char *name[3] = {"narrow", "wide", "narrow_on_first_order"};
        std::printf("%s %.3Le %.3Le %.3Lf\n", name[kind], max_norm, max_err, max_lo);
    }
    return 0;
}
