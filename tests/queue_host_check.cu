// Host-side check of the batched kernels' work queue (work_queue.cuh),
// compiled and run by test_queue_host.py: for random mixes of instances it
// builds the queue and verifies what the device side relies on --
//   * every (round, instance, unit) appears exactly once;
//   * items decode back to what was packed;
//   * round t of an instance comes after every unit of its round t - 1
//     (a unit waits only for items earlier in the queue: no deadlock);
//   * the queue is round-major, and the instances still stepping at round t
//     are a prefix of the order;
// and that over-long instances are refused.  Prints "ok" or the first
// violation.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "work_queue.cuh"

using namespace b2r;

static unsigned rnd(unsigned& s)
{
    s = s * 1664525u + 1013904223u;
    return s >> 8;
}

int main()
{
    unsigned seed = 12345;
    for (int trial = 0; trial < 200; ++trial) {
        const int n = 1 + (int)(rnd(seed) % 40);
        std::vector<int> rounds(n), units(n);
        for (int j = 0; j < n; ++j) {
            units[j] = 1 + (int)(rnd(seed) % 50);
            rounds[j] = (int)(rnd(seed) % 30);
        }
        // the queue expects instances sorted by rounds, descending
        for (int a = 0; a < n; ++a)
            for (int b = a + 1; b < n; ++b)
                if (rounds[b] > rounds[a]) {
                    std::swap(rounds[a], rounds[b]);
                    std::swap(units[a], units[b]);
                }
        std::vector<unsigned long long> items;
        if (!wq::round_major_items(rounds.data(), units.data(), n, items)) {
            printf("refused a valid mix (trial %d)\n", trial);
            return 1;
        }
        long long total = 0;
        for (int j = 0; j < n; ++j) total += (long long)rounds[j] * units[j];
        if ((long long)items.size() != total) {
            printf("size %zu != %lld (trial %d)\n", items.size(), total, trial);
            return 1;
        }
        // position of each (t, k, u); done[k][t] = units of round t of k seen so far
        std::vector<std::vector<int>> seen(n);
        for (int j = 0; j < n; ++j) seen[j].assign(rounds[j], 0);
        int last_t = 0;
        for (size_t p = 0; p < items.size(); ++p) {
            const unsigned long long x = items[p];
            const int t = (int)(x >> (wq::kItemKBits + wq::kItemUBits));
            const int k = (int)((x >> wq::kItemUBits) & ((1u << wq::kItemKBits) - 1));
            const int u = (int)(x & ((1u << wq::kItemUBits) - 1));
            if (wq::pack_item(t, k, u) != x || k >= n || t >= rounds[k] || u >= units[k]) {
                printf("bad item %llx at %zu (trial %d)\n", x, p, trial);
                return 1;
            }
            if (t < last_t) {
                printf("not round-major at %zu (trial %d)\n", p, trial);
                return 1;
            }
            last_t = t;
            if (t > 0 && seen[k][t - 1] != units[k]) {
                printf("round %d of instance %d before its round %d completed (trial %d)\n", t, k, t - 1, trial);
                return 1;
            }
            // the instances active at round t are a prefix: every earlier one is active too
            for (int j = 0; j < k; ++j)
                if (rounds[j] <= t) {
                    printf("active instances not a prefix at round %d (trial %d)\n", t, trial);
                    return 1;
                }
            if (++seen[k][t] > units[k]) {
                printf("unit listed twice (trial %d)\n", trial);
                return 1;
            }
        }
    }
    // an instance of 2^24 rounds cannot be named by an item
    {
        std::vector<int> rounds = {1 << 24}, units = {1};
        std::vector<unsigned long long> items;
        if (wq::round_major_items(rounds.data(), units.data(), 1, items)) {
            printf("accepted an instance of 2^24 rounds\n");
            return 1;
        }
    }
    // more than 2^28 items in all
    {
        std::vector<int> rounds = {1 << 15, 1 << 15}, units = {1 << 13, 1 << 13};
        std::vector<unsigned long long> items;
        if (wq::round_major_items(rounds.data(), units.data(), 2, items)) {
            printf("accepted a queue of 2^29 items\n");
            return 1;
        }
    }
    printf("ok\n");
    return 0;
}
