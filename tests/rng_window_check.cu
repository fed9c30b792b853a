// Host check of the transport kernels' random-number generator (Rng in
// egs_device.cuh): whatever the order of look-aheads (Rng::ahead), single and
// paired draws, copies and restored copies, every number equals the one a
// lazily computed Philox stream gives at that position (number n is word
// n & 3 of block n >> 2), and after ahead(k) the next k numbers need no
// block computed at the draw.  Built and run by test_rng_window.py.
#include <cstdio>
#include "egs_device.cuh"

namespace egsgpu {
static int g_draw_fills = 0;   // blocks computed at a draw (the lazy path)
static __host__ __device__ __noinline__ uint4 philox_block(uint32_t b, uint32_t s0, uint32_t s1, uint32_t k0,
                                                           uint32_t k1) {
#ifndef __CUDA_ARCH__
    ++g_draw_fills;
#endif
    uint32_t o[4];
    philox10(b, s0, s1, 0u, k0, k1, o);
    return make_uint4(o[0], o[1], o[2], o[3]);
}
}  // namespace egsgpu

using namespace egsgpu;

static float lazy_number(uint32_t seed, uint32_t hist, uint64_t sid, uint32_t n) {
    uint32_t o[4];
    philox10(n >> 2, (uint32_t)sid, (uint32_t)(sid >> 32), 0u, seed, hist, o);
    return ((float)(o[n & 3u] >> 9) + 0.5f) * (1.0f / 8388608.0f);
}

static unsigned long long lcg = 0x853c49e6748fea9bull;
static uint32_t pick(uint32_t m) {
    lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
    return (uint32_t)(lcg >> 33) % m;
}

int main() {
    long long checked = 0, covered = 0;
    for (int trial = 0; trial < 3000; ++trial) {
        const uint32_t seed = 1 + pick(1000), hist = pick(1u << 30);
        const uint64_t sid = ((uint64_t)pick(1u << 30) << 32) | pick(1u << 30);
        Rng r;
        r.init(seed, hist, sid, pick(64));
        Rng saved = r;
        int pending = 0;   // numbers still guaranteed present by the last ahead()
        for (int op = 0; op < 300; ++op) {
            const uint32_t k = pick(12);
            if (k < 3) {
                const uint32_t want = 1 + pick(13);
                r.ahead(want);
                pending = (int)want;
            } else if (k < 7) {
                const uint32_t n = r.n;
                const int before = g_draw_fills;
                const float v = r.u();
                if (v != lazy_number(seed, hist, sid, n)) { printf("draw %u differs\n", n); return 1; }
                if (pending > 0 && g_draw_fills != before) { printf("draw %u after ahead computed a block\n", n); return 2; }
                if (pending > 0) ++covered;
                --pending;
                ++checked;
            } else if (k < 10) {
                const uint32_t n = r.n;
                const int before = g_draw_fills;
                const float2 v = r.u2();
                if (v.x != lazy_number(seed, hist, sid, n) || v.y != lazy_number(seed, hist, sid, n + 1)) {
                    printf("pair %u differs\n", n);
                    return 1;
                }
                if (pending > 1 && g_draw_fills != before) { printf("pair %u after ahead computed a block\n", n); return 2; }
                pending -= 2;
                checked += 2;
            } else if (k == 10) {   // a copy continues the stream but holds no window
                Rng c = r;
                r = c;
                pending = 0;
            } else {                 // go back to an earlier copy (its position), or take one
                if (pick(2)) { r = saved; pending = 0; }
                else saved = r;
            }
        }
    }
    printf("ok %lld numbers, %lld drawn from a look-ahead\n", checked, covered);
    return 0;
}
