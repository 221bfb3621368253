// CPU checks of the job server's host-side policy (server_policy.hpp):
// first-come-first-served admission under slots and bytes, round length,
// snapshot schedule and nearest-rank percentiles.  Prints "ok" or the first
// failed check and exits non-zero.
#include <cstdio>
#include <vector>

#include "server_policy.hpp"

using namespace nbgb;

#define CHECK(c)                                                     \
    do {                                                             \
        if (!(c)) {                                                  \
            std::printf("failed: %s (line %d)\n", #c, __LINE__);     \
            return 1;                                                \
        }                                                            \
    } while (0)

int main() {
    // admission: bytes and slots
    Admission a(100, 2);
    CHECK(a.can_ever_fit(100) && !a.can_ever_fit(101));
    CHECK(a.fits(60));
    a.reserve(60);
    CHECK(!a.fits(50) && a.fits(40));
    a.reserve(40);
    CHECK(a.in_use() == 100 && a.jobs() == 2 && !a.fits(0));  // no slot left
    a.release(60);
    CHECK(a.fits(60) && !a.fits(61));
    a.release(40);
    CHECK(a.in_use() == 0 && a.jobs() == 0 && a.peak() == 100 && a.peak_jobs() == 2);

    // first come first served: simulate a queue where the head does not fit
    // yet; a later small job must not overtake it
    {
        Admission q(100, 8);
        std::vector<int64_t> queue = {70, 50, 10};
        std::vector<int> order;
        q.reserve(40);  // a running job
        size_t head = 0;
        auto step = [&] {
            while (head < queue.size() && q.fits(queue[head])) {
                q.reserve(queue[head]);
                order.push_back((int)head);
                ++head;
            }
        };
        step();
        CHECK(order.empty());  // 70 waits for the running 40; 10 may not pass it
        q.release(40);
        step();
        CHECK(order.size() == 1 && order[0] == 0);  // 70 in; 50 waits
        q.release(70);
        step();
        CHECK(order.size() == 3 && order[1] == 1 && order[2] == 2);
    }

    // rounds: the snapshot period, cut short when every job ends sooner
    CHECK(round_steps({35, 7}, 10) == 10);
    CHECK(round_steps({5, 3}, 10) == 5);
    CHECK(round_steps({500}, 0) == 10);
    CHECK(round_steps({4}, 0) == 4);
    CHECK(round_steps({}, 10) == 0);

    // a 35-step job in rounds of 10: snapshots at 10, 20, 30, result at 35
    {
        std::vector<int> snaps;
        int done = 0;
        while (done < 35) {
            done = steps_after(done, 35, round_steps({35 - done}, 10));
            if (snapshot_due(done, 35, 10)) snaps.push_back(done);
        }
        CHECK(done == 35 && snaps.size() == 3 && snaps[0] == 10 && snaps[2] == 30);
        CHECK(!snapshot_due(40, 40, 10));  // the last state is the result
        CHECK(!snapshot_due(10, 40, 0));
    }

    // nearest-rank percentiles
    std::vector<double> v;
    for (int i = 1; i <= 100; ++i) v.push_back((double)(101 - i));
    CHECK(percentile(v, 50) == 50.0);
    CHECK(percentile(v, 99) == 99.0);
    CHECK(percentile(v, 100) == 100.0);
    CHECK(percentile(v, 0) == 1.0);
    CHECK(percentile({}, 50) == 0.0);
    CHECK(percentile({3.0}, 99) == 3.0);
    std::printf("ok\n");
    return 0;
}
