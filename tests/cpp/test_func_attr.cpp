// CPU test of FuncAttrCache (g-ls3u_gb300/csrc/func_attr.hpp): the record of
// raised shared-memory limits is kept per (kernel, device), never lowered,
// and consistent when many threads make their first launch at once.
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "func_attr.hpp"

static int failures = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAILED line %d: %s\n", __LINE__, #c);     \
            failures++;                                            \
        }                                                          \
    } while (0)

int main()
{
    glsu::FuncAttrCache c;
    int k1 = 0, k2 = 0;  // stand-ins for two kernels' addresses
    CHECK(c.needs(&k1, 0, 1000));
    c.done(&k1, 0, 1000);
    CHECK(!c.needs(&k1, 0, 1000));
    CHECK(!c.needs(&k1, 0, 500));
    CHECK(c.needs(&k1, 0, 2000));  // a larger limit is raised again
    CHECK(c.needs(&k1, 1, 1000));  // another device starts from nothing
    CHECK(c.needs(&k2, 0, 1000));  // another kernel too
    c.done(&k1, 0, 500);           // never lowered
    CHECK(c.recorded(&k1, 0) == 1000);

    // 16 threads x 8 devices: every (kernel, device) is raised, and the
    // records end at the largest limit any thread asked for
    glsu::FuncAttrCache m;
    std::atomic<int> raises{0};
    std::vector<std::thread> th;
    for (int t = 0; t < 16; t++)
        th.emplace_back([&, t]() {
            for (int dev = 0; dev < 8; dev++) {
                const int bytes = 1024 * (1 + (t + dev) % 4);
                if (m.needs(&k2, dev, bytes)) {
                    raises++;
                    m.done(&k2, dev, bytes);
                }
            }
        });
    for (auto &x : th) x.join();
    for (int dev = 0; dev < 8; dev++) CHECK(m.recorded(&k2, dev) == 4096);
    CHECK(raises.load() >= 8);
    if (failures) return 1;
    std::printf("func_attr ok (%d raises)\n", raises.load());
    return 0;
}
