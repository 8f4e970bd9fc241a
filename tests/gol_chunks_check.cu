// Host-side check of the Game-of-Life pass's z-chunk model (gol.h,
// gol_period_chunks), compiled and run by test_queue_host.py: the count
// measured best on the 256^3 torus in 2 x 2 x 2 blocks (19 chunks of the 128
// planes, 32 tiles, 152 SMs, 5 CTAs per SM at most, 4 generations) is the one
// picked; the pick never makes more CTAs than fit at once and keeps at least
// minper per SM on average where the block allows; a block too large for one
// wave gets one chunk.  Prints "ok" or the first violation.
#include <cstdio>

#include "gol.h"

using namespace b2r;

int main()
{
    const int c = gol_period_chunks(32, 128, 4, 152, 5, 3);
    if (c != 19) {
        printf("256^3 torus: picked %d chunks, measured best 19\n", c);
        return 1;
    }
    unsigned s = 7;
    for (int trial = 0; trial < 2000; ++trial) {
        s = s * 1664525u + 1013904223u;
        const long long tiles = 1 + (s >> 8) % 300;
        s = s * 1664525u + 1013904223u;
        const int nz = 1 + (int)((s >> 8) % 600);
        const int ng = 1 + (int)((s >> 4) % 4);
        const int cap = 1 + (int)((s >> 12) % 8);
        const int sms = 152, minper = 3;
        const int k = gol_period_chunks(tiles, nz, ng, sms, cap, minper);
        if (k < 1 || k > nz) {
            printf("chunks %d outside 1..%d\n", k, nz);
            return 1;
        }
        const long long ctas = tiles * k;
        if (k > 1 && ctas > (long long)sms * cap) {
            printf("%lld CTAs do not fit (%d per SM)\n", ctas, cap);
            return 1;
        }
        // where some count fits at once and reaches minper per SM, the pick does
        bool reachable = false;
        for (int cc = 1; cc <= nz; ++cc) {
            const long long n = tiles * cc;
            if (n > (long long)sms * cap) break;
            if (n >= (long long)minper * sms) reachable = true;
        }
        if (reachable && ctas < (long long)minper * sms) {
            printf("picked %lld CTAs below %d per SM although reachable\n", ctas, minper);
            return 1;
        }
        if (tiles > (long long)sms * cap && k != 1) {
            printf("a block beyond one wave split into %d chunks\n", k);
            return 1;
        }
    }
    printf("ok\n");
    return 0;
}
