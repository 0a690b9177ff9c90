// Host-only check of ftl::AttrRegistry (the per-device bookkeeping behind
// ensure_smem): a fake setter stands in for cudaFuncSetAttribute.
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "attr_registry.h"

static int failures = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);       \
            ++failures;                                            \
        }                                                          \
    } while (0)

int main() {
    ftl::AttrRegistry reg;
    int k1 = 0, k2 = 0;  // two "kernels" (only their addresses matter)
    std::vector<std::pair<int, int>> calls;  // (device, bytes) passed to the setter
    int dev = 0;
    auto setter = [&](int b) {
        calls.emplace_back(dev, b);
        return 0;
    };

    // first use on device 0 sets; a repeat or a smaller request does not
    dev = 0;
    CHECK(reg.ensure(&k1, 0, 100000, setter) == 0);
    CHECK(reg.ensure(&k1, 0, 100000, setter) == 0);
    CHECK(reg.ensure(&k1, 0, 60000, setter) == 0);
    CHECK(calls.size() == 1);
    // the same kernel on device 1 must be set again (attributes are per device)
    dev = 1;
    CHECK(reg.ensure(&k1, 1, 100000, setter) == 0);
    CHECK(calls.size() == 2 && calls[1].first == 1);
    // a larger request raises the limit; another kernel is independent
    CHECK(reg.ensure(&k1, 1, 200000, setter) == 0);
    CHECK(calls.size() == 3 && reg.limit(&k1, 1) == 200000 && reg.limit(&k1, 0) == 100000);
    CHECK(reg.ensure(&k2, 1, 100000, setter) == 0);
    CHECK(calls.size() == 4);
    // a refused setting is reported and not recorded, so the next call retries
    auto refuse = [&](int) { return 7; };
    CHECK(reg.ensure(&k2, 2, 150000, refuse) == 7);
    CHECK(reg.limit(&k2, 2) == 0);
    CHECK(reg.ensure(&k2, 2, 150000, setter) == 0 && reg.limit(&k2, 2) == 150000);

    // many threads on many devices: each (kernel, device) is set exactly once
    ftl::AttrRegistry reg2;
    std::atomic<int> sets[8];
    for (auto &s : sets) s = 0;
    std::vector<std::thread> th;
    for (int t = 0; t < 16; ++t)
        th.emplace_back([&, t] {
            for (int it = 0; it < 1000; ++it) {
                const int d = (t + it) % 8;
                reg2.ensure(&k1, d, 120000, [&](int) {
                    sets[d]++;
                    return 0;
                });
            }
        });
    for (auto &x : th) x.join();
    for (int d = 0; d < 8; ++d) CHECK(sets[d] == 1);

    if (failures == 0) std::printf("attr_registry ok\n");
    return failures == 0 ? 0 : 1;
}
