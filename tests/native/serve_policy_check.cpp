// Unit checks of the serving runtime's host policy (vship_gb300/csrc/serve_policy.h): admission,
// the LRU source cache with pinning, FIFO continuous batching. Prints one line per check and
// exits non-zero on the first failure.
#include "../../vship_gb300/csrc/serve_policy.h"

#include <cstdio>
#include <cstdlib>

using namespace vship;

#define CHECK(cond)                                                 \
    do {                                                            \
        if (!(cond)) {                                              \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond); \
            std::exit(1);                                           \
        }                                                           \
    } while (0)

struct Req {
    int pairs;
    uint64_t charge;
};

int main() {
    // charges: 12 and 31 FP32 planes per pair
    CHECK(serve_charge_per_pair(SERVE_SSIMU2, 3840, 2160) == 48ull * 3840 * 2160);
    CHECK(serve_charge_per_pair(SERVE_BUTTERAUGLI, 1920, 1080) == 124ull * 1920 * 1080);
    std::printf("ok charges\n");

    Admission a(100);
    CHECK(a.fits_alone(100) && !a.fits_alone(101));
    CHECK(a.try_charge(60) && !a.try_charge(41) && a.try_charge(40));
    CHECK(a.used() == 100 && a.peak() == 100);
    a.release(60);
    CHECK(a.used() == 40 && a.try_charge(60));
    std::printf("ok admission\n");

    SourceCache<int> c(100);
    std::vector<int> ev;
    const SourceKey k1{0, 0, 1}, k2{0, 0, 2}, k3{0, 0, 3}, k4{1, 0, 1};
    CHECK(c.insert(k1, 11, 40, &ev) && c.insert(k2, 22, 40, &ev) && ev.empty());
    int v = 0;
    CHECK(!c.acquire(k3, &v) && c.misses() == 1);
    // k1 and k2 pinned by their inserts: no room for k3
    CHECK(!c.insert(k3, 33, 40, &ev) && ev.empty() && c.size() == 2);
    c.unpin(k1);
    c.unpin(k2);
    CHECK(c.acquire(k1, &v) && v == 11 && c.hits() == 1);  // k1 now most recent
    c.unpin(k1);
    CHECK(c.insert(k3, 33, 40, &ev) && ev.size() == 1 && ev[0] == 22);  // least recent (k2) goes
    CHECK(c.pins(k2) == -1 && c.bytes() == 80 && c.evictions() == 1);
    // same key, other metric: a different entry
    CHECK(!c.acquire(k4, &v));
    ev.clear();
    CHECK(c.insert(k4, 44, 20, &ev) && ev.empty() && c.bytes() == 100);
    // pinned entries survive; an insert that cannot fit changes nothing
    CHECK(c.acquire(k1, &v));
    c.unpin(k3);
    c.unpin(k4);
    CHECK(c.insert(SourceKey{0, 1, 9}, 99, 60, &ev) && ev.size() == 2);
    CHECK(c.pins(k1) == 1 && c.size() == 2);
    ev.clear();
    CHECK(!c.insert(SourceKey{0, 1, 10}, 5, 101, &ev) && ev.empty());
    int e = 0;
    CHECK(c.erase(k1, &e) && e == 11 && c.bytes() == 60);
    std::printf("ok cache\n");

    // batching: FIFO, stops at the first request that does not fit, max pairs per batch
    std::deque<Req*> q;
    Req r[5] = {{4, 10}, {8, 20}, {2, 50}, {1, 5}, {16, 10}};
    for (auto& x : r) q.push_back(&x);
    Admission b(60);
    auto ch = [](Req* x) { return x->charge; };
    auto pp = [](Req* x) { return x->pairs; };
    auto bt = form_batch(q, b, 16, ch, pp);
    CHECK(bt.size() == 2 && bt[0] == &r[0] && bt[1] == &r[1] && b.used() == 30);  // r[2] waits (50 > 30 left)
    CHECK(form_batch(q, b, 16, ch, pp).empty());                                 // no overtaking by r[3]
    b.release(30);
    bt = form_batch(q, b, 16, ch, pp);
    CHECK(bt.size() == 2 && bt[0] == &r[2] && bt[1] == &r[3]);  // r[4]: 16 more pairs exceed 16
    b.release(55);
    bt = form_batch(q, b, 16, ch, pp);
    CHECK(bt.size() == 1 && bt[0] == &r[4] && q.empty());  // alone it may fill the batch
    std::printf("ok batching\n");
    return 0;
}
