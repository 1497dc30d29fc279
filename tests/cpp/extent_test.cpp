// Host-only checks of the page allocator behind scene pools (extent.hpp): first
// fit, merging of freed runs, high-water mark, fits_now/fits_ever, and a random
// admit/retire sequence checked against a brute-force page map.  Prints "ok".
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>

#include "../../twoscalesplit_gb300/csrc/extent.hpp"

#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "check failed line %d: %s\n", __LINE__, #c); \
            return 1;                                                     \
        }                                                                 \
    } while (0)

int main() {
    tss::ExtentSet e(1000, 64);  // 15 pages of 64 = 960 units
    CHECK(e.capacity() == 960);
    int64_t a, b, c, d;
    CHECK(e.alloc(100, &a) && a == 0);   // 2 pages
    CHECK(e.alloc(64, &b) && b == 128);  // 1 page
    CHECK(e.alloc(1, &c) && c == 192);
    CHECK(e.high_water() == 256);
    CHECK(e.free_units() == 960 - 256);
    CHECK(e.release(b));
    CHECK(!e.release(b));                // double free refused
    CHECK(e.alloc(65, &d) && d == 256);  // 2 pages do not fit the 1-page hole
    CHECK(e.alloc(10, &b) && b == 128);  // first fit takes the hole
    CHECK(e.release(a) && e.release(b) && e.release(c));
    CHECK(e.high_water() == 384);        // d still there
    CHECK(e.alloc(192, &a) && a == 0);   // freed runs merged into [0, 256)
    CHECK(e.release(d) && e.release(a));
    CHECK(e.high_water() == 0 && e.free_units() == 960);
    CHECK(e.fits_ever(960) && !e.fits_ever(961));
    CHECK(e.alloc(960, &a) && !e.fits_now(1) && e.release(a));

    // random sequence against a page map
    std::mt19937 rng(7);
    tss::ExtentSet r(64 * 512, 64);
    std::vector<int> owner(512, -1);
    std::map<int, std::pair<int64_t, int64_t>> live;  // id -> (start, len)
    int next_id = 0;
    for (int it = 0; it < 20000; ++it) {
        if (live.empty() || rng() % 3) {
            int64_t n = 1 + rng() % (64 * 40);
            int64_t at;
            bool ok = r.alloc(n, &at);
            // brute force: lowest run of free pages that fits
            const int64_t pages = (n + 63) / 64;
            int64_t best = -1, run = 0;
            for (int p = 0; p < 512; ++p) {
                run = owner[p] < 0 ? run + 1 : 0;
                if (run == pages) {
                    best = p - pages + 1;
                    break;
                }
            }
            CHECK(ok == (best >= 0));
            if (ok) {
                CHECK(at == best * 64);
                for (int64_t p = best; p < best + pages; ++p) owner[p] = next_id;
                live[next_id++] = {at, pages * 64};
            }
        } else {
            auto itl = live.begin();
            std::advance(itl, rng() % live.size());
            CHECK(r.release(itl->second.first));
            for (int64_t p = itl->second.first / 64; p < (itl->second.first + itl->second.second) / 64; ++p) owner[p] = -1;
            live.erase(itl);
        }
        int64_t hw = 0, fr = 0;
        for (int p = 0; p < 512; ++p) {
            if (owner[p] >= 0) hw = (p + 1) * 64;
            else fr += 64;
        }
        CHECK(r.high_water() == hw && r.free_units() == fr);
    }
    std::printf("ok\n");
    return 0;
}
