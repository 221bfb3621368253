// Host-side sizing rules of the tree and batched-system buffers (no device
// code runs): the number of top octree levels built from region counts, the
// bodies per build block of a batch, the tree capacity of a batched system,
// and the layout of a system's buffers (256-byte alignment, the top-level
// tables present exactly when a tree has top levels).  Prints "ok".
#include <cstdint>
#include <cstdio>

#include "sysmem.cuh"

using namespace nbgb;

static int fails = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); \
            ++fails;                                               \
        }                                                          \
    } while (0)

static bool aligned256(const void *p) { return ((uintptr_t)p & 255) == 0; }

int main() {
    // about 8 bodies or more per region of the deepest top level, 2..5 levels
    CHECK(top_levels_for(0) == 0);
    CHECK(top_levels_for(511) == 0);
    CHECK(top_levels_for(512) == 2);
    CHECK(top_levels_for(4095) == 2);
    CHECK(top_levels_for(4096) == 3);
    CHECK(top_levels_for(32767) == 3);
    CHECK(top_levels_for(32768) == 4);
    CHECK(top_levels_for(262143) == 4);
    CHECK(top_levels_for(262144) == 5);
    CHECK(top_levels_for(1 << 24) == kTopMaxLevels);
    // batched trees count in 4096 shared-memory bins at most
    CHECK(batch_top_levels_for(262144) == 4);
    CHECK(batch_top_levels_for(4096) == 3);
    CHECK(batch_top_levels_for(100) == 0);
    CHECK((1 << (3 * kBatchTopMaxLevels)) == 4096);
    CHECK(kTopInner == 8 + 64 + 512 + 4096);

    // bodies per build block of a batched tree
    CHECK(batch_chunk(1000, 1000) == 1024);
    CHECK(batch_chunk(1 << 19, 1 << 19) == 4096);
    CHECK(batch_chunk(1000, 4LL << 20) == 4096);

    // tree capacity of a batched system: max(2N, 4096) rounded up to 16
    CHECK(sysmem_default_capacity(10) == 4096);
    CHECK(sysmem_default_capacity(100001) == 200016);

    // a system's buffers, laid out from a fake base: every array 256-byte
    // aligned and inside [base, base + bytes)
    for (int n : {1000, 5000, 300000}) {
        for (int quad = 0; quad < 2; ++quad) {
            SysMem m;
            m.n = n;
            m.tree = true;
            m.quad = quad != 0;
            m.cap = sysmem_default_capacity(n);
            const size_t bytes = sysmem_layout(m, nullptr);
            char *base = reinterpret_cast<char *>((uintptr_t)1 << 40);  // never dereferenced
            SysMem v = m;
            CHECK(sysmem_layout(v, base) == bytes);
            const void *arrays[] = {v.body[0], v.body[1], v.vel, v.acc, v.parent, v.child, v.wchild, v.wpm,
                                    v.cell_pm, v.count, v.start, v.arrive, v.sorted};
            for (const void *a : arrays) {
                CHECK(a != nullptr && aligned256(a));
                CHECK((const char *)a >= base && (const char *)a < base + bytes);
            }
            CHECK((v.cell_q != nullptr) == m.quad && (v.wqa != nullptr) == m.quad);
            CHECK(v.top_levels == batch_top_levels_for(n));
            int *counts = nullptr;
            size_t count_bytes = 0;
            sysmem_top_counts(v, &counts, &count_bytes);
            if (v.top_levels) {
                CHECK(counts == v.top && aligned256(counts));
                CHECK(count_bytes == sizeof(int) << (3 * v.top_levels));
                CHECK((char *)counts + 2 * count_bytes <= base + bytes);  // counts, then start entries
            } else {
                CHECK(counts == nullptr && count_bytes == 0);
            }
        }
    }
    // a direct-sum system has no tree buffers
    SysMem d;
    d.n = 5000;
    d.tree = false;
    char *base = reinterpret_cast<char *>((uintptr_t)1 << 40);
    sysmem_layout(d, base);
    CHECK(d.child == nullptr && d.top == nullptr && d.body[0] != nullptr);

    if (fails == 0) std::printf("ok\n");
    return fails == 0 ? 0 : 1;
}
