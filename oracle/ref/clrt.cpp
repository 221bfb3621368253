/*
 * clrt.cpp -- TEST INFRASTRUCTURE (oracle). Never linked into the product.
 *
 * A tiny single-threaded "CPU OpenCL device" for the reference's kernels:
 * every work-item of an NDRange is a ucontext coroutine, all work-groups are
 * live at once (the reference's build_tree / saturate_tree spin on values
 * that other work-groups produce), and the scheduler runs round-robin:
 * groups in ascending order, work-items of a group in DESCENDING local id.
 *
 * Descending order inside a group matters for calculate_forces.cl, where
 * lane 0 of a 16-lane warp ("sBase") writes the shared stack slot that the
 * other lanes have just read: on SIMT hardware every lane reads before lane
 * 0 writes, and running lane 0 last between two sync points reproduces that.
 *
 * Barrier semantics: a work-item at a barrier (or work_group_all) waits until
 * every work-item of its group that has not finished is also at a barrier.
 * Finished work-items count as arrived, so the reference's barriers inside
 * divergent loops (build_tree.cl:159) cannot deadlock here.
 *
 * Local memory: the statics of the "clref_local" section are saved/restored
 * whenever the scheduler moves from one work-group to another.
 */
#include <ucontext.h>
#include <sys/mman.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

extern "C" char __start_clref_local[] __attribute__((weak));
extern "C" char __stop_clref_local[] __attribute__((weak));

namespace {

enum ItemState { READY = 0, WAITING = 1, DONE = 2 };

struct Item {
    ucontext_t ctx;
    size_t gid, lid, grp;
    int state;
    int collective;  // waiting inside work_group_all
    int pred;
    int result;
};

struct Launch {
    size_t global = 0, local = 0, ngroups = 0;
    std::vector<Item> items;
    const std::function<void()> *body = nullptr;
    ucontext_t sched;
    Item *cur = nullptr;
    char *stacks = nullptr;
    size_t stack_bytes = 0, stack_total = 0;
};

Launch *g_launch = nullptr;
long g_round_cap = 200000000L;

void item_entry() {
    Launch *L = g_launch;
    (*L->body)();
    L->cur->state = DONE;
    // returning resumes uc_link (the scheduler)
}

}  // namespace

extern "C" {

size_t clref_get_global_id(unsigned) { return g_launch->cur->gid; }
size_t clref_get_local_id(unsigned) { return g_launch->cur->lid; }
size_t clref_get_group_id(unsigned) { return g_launch->cur->grp; }
size_t clref_get_global_size(unsigned) { return g_launch->global; }
size_t clref_get_local_size(unsigned) { return g_launch->local; }
size_t clref_get_num_groups(unsigned) { return g_launch->ngroups; }

void clref_yield(void) {
    Item *it = g_launch->cur;
    swapcontext(&it->ctx, &g_launch->sched);
}

void clref_barrier(void) {
    Item *it = g_launch->cur;
    it->state = WAITING;
    it->collective = 0;
    swapcontext(&it->ctx, &g_launch->sched);
}

int clref_work_group_all(int p) {
    Item *it = g_launch->cur;
    it->state = WAITING;
    it->collective = 1;
    it->pred = p;
    swapcontext(&it->ctx, &g_launch->sched);
    return it->result;
}

void clref_set_round_cap(long cap) { g_round_cap = cap; }

/* Run `body` for every work-item of a 1-D NDRange.  Returns 0 on success,
 * -1 when the round cap is exceeded (a livelock/deadlock of the kernel). */
int clref_launch(size_t global, size_t local, const std::function<void()> *body) {
    if (local == 0 || global % local != 0) return -2;
    Launch L;
    L.global = global;
    L.local = local;
    L.ngroups = global / local;
    L.body = body;
    L.items.resize(global);
    L.stack_bytes = 64 * 1024;
    L.stack_total = L.stack_bytes * global;
    void *mem = mmap(nullptr, L.stack_total, PROT_READ | PROT_WRITE,
                     MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (mem == MAP_FAILED) return -3;
    L.stacks = (char *)mem;

    Launch *prev = g_launch;
    g_launch = &L;
    for (size_t i = 0; i < global; ++i) {
        Item &it = L.items[i];
        it.gid = i;
        it.lid = i % local;
        it.grp = i / local;
        it.state = READY;
        it.collective = 0;
        it.pred = 1;
        it.result = 1;
        getcontext(&it.ctx);
        it.ctx.uc_stack.ss_sp = L.stacks + i * L.stack_bytes;
        it.ctx.uc_stack.ss_size = L.stack_bytes;
        it.ctx.uc_link = &L.sched;
        makecontext(&it.ctx, (void (*)())item_entry, 0);
    }

    const size_t lm_bytes = (__start_clref_local && __stop_clref_local)
                                ? (size_t)(__stop_clref_local - __start_clref_local) : 0;
    std::vector<std::vector<char>> lmem(L.ngroups, std::vector<char>(lm_bytes, 0));
    long mapped = -1;

    size_t live = global;
    long rounds = 0;
    int rc = 0;
    while (live > 0) {
        for (size_t g = 0; g < L.ngroups; ++g) {
            Item *base = &L.items[g * local];
            bool any_ready = false;
            for (size_t l = 0; l < local; ++l)
                if (base[l].state == READY) { any_ready = true; break; }
            if (any_ready) {
                if (lm_bytes && mapped != (long)g) {
                    if (mapped >= 0) memcpy(lmem[mapped].data(), __start_clref_local, lm_bytes);
                    memcpy(__start_clref_local, lmem[g].data(), lm_bytes);
                    mapped = (long)g;
                }
                for (size_t l = local; l-- > 0;) {
                    Item &it = base[l];
                    if (it.state != READY) continue;
                    L.cur = &it;
                    swapcontext(&L.sched, &it.ctx);
                    if (it.state == DONE) --live;
                }
            }
            // release the group's barrier when no member is still running
            bool waiting = false, running = false;
            int all = 1;
            for (size_t l = 0; l < local; ++l) {
                if (base[l].state == READY) running = true;
                else if (base[l].state == WAITING) {
                    waiting = true;
                    if (base[l].collective && !base[l].pred) all = 0;
                }
            }
            if (waiting && !running) {
                for (size_t l = 0; l < local; ++l)
                    if (base[l].state == WAITING) {
                        base[l].state = READY;
                        base[l].result = all;
                    }
            }
        }
        if (++rounds > g_round_cap) { rc = -1; break; }
    }
    if (lm_bytes && mapped >= 0) memcpy(lmem[mapped].data(), __start_clref_local, lm_bytes);
    munmap(L.stacks, L.stack_total);
    g_launch = prev;
    return rc;
}

}  // extern "C"
