// force_device.cuh -- the Barnes-Hut force walk of one warp group, shared
// by the single-system kernel (k_force.cu) and the batched one (k_batch.cu).
// (calculate_force_local, kernels/calculate_forces.cl:4-185.)
//
// One warp owns 32 consecutive bodies of the in-order sort (spatial
// neighbours).  The warp keeps one shared stack of cells still to open.  Each
// round pops up to kBatch = 8 cells and opens them together: lane L loads
// child slot L%8 of popped cells L/8 and 4 + L/8 -- index, packed {x,y,z,m}
// and (with quadrupoles) moments, coalesced 128-byte lines, one memory round
// trip for up to 64 children -- and the warp stages them compacted into a
// body list and a cell list, in pop and slot order.  Eight cells a round
// instead of four halve the rounds and their fixed cost (4M workload: force
// 14.12 -> 13.71 ms; 512-system batch 49.09 -> 47.97 ms per step).  Bodies are always accumulated; a cell is accumulated
// when EVERY lane accepts it (__all_sync of d^2 >= dq[level], the reference's
// work_group_all at :121, over a real 32-lane warp), otherwise it is pushed.
// Softened gravity F = m rsqrt(d^2)^3 (MUFU rsqrt), d^2 = |d|^2 + eps^2 as
// FMAs; accepted cells optionally add their traceless quadrupole.
//
// Stack bound: kBatch cells are popped only while the stack holds at most
// kBatchBelow entries, so a batch leaves at most kBatchBelow - 1 + 8*kBatch
// entries; beyond that the walk pops one cell at a time (depth first), which
// adds at most 7 pending siblings per tree level: at most 127 + 64 + 7*63 + 1
// = 633 <= kStack entries for any tree of fewer than kMaxDepth levels.
// Entries pack (level << 26) | node.
//
// The integrator writes the next position buffer, so every force of the step
// sees step-start positions (the reference integrates in place while other
// work-items still read positions, :159-180).
#pragma once
#include "nbgb_internal.cuh"

namespace nbgb {

constexpr int kForceWarps = 4;
constexpr int kForceThreads = kForceWarps * 32;
constexpr int kStack = 640;
constexpr int kBatch = 8;
static_assert(kBatch == 8, "a lane loads slot L%8 of popped cells L/8 and 4 + L/8");
constexpr int kBatchBelow = 128;  // batch pops only while the stack holds at most this many
constexpr int kNodeBits = 26;
constexpr int kNodeMask = (1 << kNodeBits) - 1;

template <int kMethod>
__device__ __forceinline__ void integrate_body(const DevSim &s, const StepParams &p, int b, const float4 P, float ax,
                                               float ay, float az) {
    const float dt = p.dt;
    const float4 v = s.vel[b];
    float4 x = P, vo = v;
    if constexpr (kMethod == 2) {  // Euler (calculate_forces.cl:168-181)
        vo.x = __fadd_rn(v.x, __fmul_rn(ax, dt));
        vo.y = __fadd_rn(v.y, __fmul_rn(ay, dt));
        vo.z = __fadd_rn(v.z, __fmul_rn(az, dt));
        x.x = __fadd_rn(P.x, __fmul_rn(vo.x, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(vo.y, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(vo.z, dt));
        s.acc[b] = make_float4(ax, ay, az, 0.0f);
    } else if constexpr (kMethod == 1) {  // "Leapfrog" as written (:152-167): acc read, not written
        const float4 ap = s.acc[b];
        const float hx = __fadd_rn(v.x, __fmul_rn(__fmul_rn(ap.x, dt), 0.5f));
        const float hy = __fadd_rn(v.y, __fmul_rn(__fmul_rn(ap.y, dt), 0.5f));
        const float hz = __fadd_rn(v.z, __fmul_rn(__fmul_rn(ap.z, dt), 0.5f));
        x.x = __fadd_rn(P.x, __fmul_rn(hx, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(hy, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(hz, dt));
        vo.x = __fadd_rn(hx, __fmul_rn(__fmul_rn(ax, dt), 0.5f));
        vo.y = __fadd_rn(hy, __fmul_rn(__fmul_rn(ay, dt), 0.5f));
        vo.z = __fadd_rn(hz, __fmul_rn(__fmul_rn(az, dt), 0.5f));
    } else if constexpr (kMethod == 3) {  // kick-drift-kick, velocities at half steps
        const float h = p.kdk_primed ? dt : __fmul_rn(dt, 0.5f);
        vo.x = __fadd_rn(v.x, __fmul_rn(ax, h));
        vo.y = __fadd_rn(v.y, __fmul_rn(ay, h));
        vo.z = __fadd_rn(v.z, __fmul_rn(az, h));
        x.x = __fadd_rn(P.x, __fmul_rn(vo.x, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(vo.y, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(vo.z, dt));
        s.acc[b] = make_float4(ax, ay, az, 0.0f);
    } else {  // any other method value moves nothing (the as-wired reference)
    }
    s.vel[b] = vo;
    s.body_next[b] = x;
}

// TwoSum (Knuth): hi + t = s + e exactly; e goes to the low word.
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float t) {
    const float s = __fadd_rn(hi, t);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(t, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

// Shared-memory staging of one warp.
struct WarpStage {
    int *stack;     // kStack packed cell entries
    float4 *bpm;    // 8 * kBatch staged child bodies {x,y,z,m}
    float4 *cpm;    // 8 * kBatch staged child cells {x,y,z,m}
    float4 *cmeta;  // {q_xz, q_yz, threshold, packed child}
    float4 *cqa;    // {q_xx, q_yy, q_zz, q_xy}
};

// The nc cells staged this round, in order: accumulated into (sx, sy, sz)
// when every lane accepts, else pushed.  kChecked: the round's pushes may
// fill the stack, so each push tests for room and a cell beyond the bound
// is dropped with the depth status (the walk's result is then discarded);
// otherwise every push fits and the test is left out of the loop.
template <bool kQuad, bool kChecked>
__device__ __forceinline__ void cell_list(const float4 *cpm, const float4 *cmeta, const float4 *cqa, int nc,
                                          const float4 P, float eps2, float &sx, float &sy, float &sz, int *stack,
                                          int &sp, unsigned &n_drop, int lane, Ctrl *ctrl) {
    for (int k = 0; k < nc; ++k) {
        const float4 q = cpm[k];
        const float4 mt = cmeta[k];
        const float dx = q.x - P.x, dy = q.y - P.y, dz = q.z - P.z;
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
        if (__all_sync(0xffffffffu, d2 >= mt.z)) {
            const float r = rsqrt_fast(d2);
            const float r2 = r * r;
            if constexpr (kQuad) {
                // m d / r^3 + 2.5 (d.Q.d) d / r^7 - Q d / r^5
                //   = (d (m d^2 + 2.5 (d.Q.d) / r^2) - Q d) / r^5, with r^-2 = d^2:
                // 24 FP32 operations instead of 26
                const float4 Q = cqa[k];  // xx yy zz xy; mt.x = xz, mt.y = yz
                const float qx = fmaf(mt.x, dz, fmaf(Q.w, dy, Q.x * dx));
                const float qy = fmaf(mt.y, dz, fmaf(Q.y, dy, Q.w * dx));
                const float qz = fmaf(Q.z, dz, fmaf(mt.y, dy, mt.x * dx));
                const float sq = fmaf(dz, qz, fmaf(dy, qy, dx * qx));
                const float r5 = r * (r2 * r2);
                const float t = fmaf(2.5f * sq, r2, q.w * d2);
                sx = fmaf(fmaf(dx, t, -qx), r5, sx);
                sy = fmaf(fmaf(dy, t, -qy), r5, sy);
                sz = fmaf(fmaf(dz, t, -qz), r5, sz);
            } else {
                const float F = q.w * (r * r2);
                sx = fmaf(dx, F, sx);
                sy = fmaf(dy, F, sy);
                sz = fmaf(dz, F, sz);
            }
        } else if (!kChecked || sp < kStack) {
            if (lane == 0) stack[sp] = __float_as_int(mt.w);
            ++sp;
        } else {  // outside the stack bound: never overrun shared memory
            ++n_drop;
            if (lane == 0) set_status(ctrl, kStDepth, kStack);
        }
    }
}

// Walk of warp group g of system s (dq: its 64 thresholds), with the fused
// integrator.  All 32 lanes call it together.
template <int kMethod, bool kComp, bool kEpsZero, bool kQuad>
__device__ __forceinline__ void force_group(const DevSim &s, const StepParams &p, const float *dq, int g, int lane,
                                            const WarpStage &ws) {
    Ctrl *ctrl = s.ctrl;
    const int n = s.n, root = n + s.cap;
    int *stack = ws.stack;
    float4 *bpm = ws.bpm, *cpm = ws.cpm, *cmeta = ws.cmeta, *cqa = ws.cqa;
    const float eps2 = __fmul_rn(p.eps, p.eps);
    const int cidx = lane >> 3, slot = lane & 7;
    const unsigned below = (1u << lane) - 1u;
    const int sidx = g * 32 + lane;
    const bool valid = sidx < n;
    // a lane past the end takes lane 0's body: its votes copy lane 0's,
    // so the warp vote needs no validity test; its result is discarded
    const int b = s.sorted[valid ? sidx : g * 32];
    const float4 P = s.body_cur[b];
    float ax = 0.0f, ay = 0.0f, az = 0.0f, lx = 0.0f, ly = 0.0f, lz = 0.0f;
    unsigned n_body = 0, n_cell = 0, n_open = 0, n_drop = 0;  // n_cell: staged cells
    int sp = 1;
    if (lane == 0) stack[0] = root;  // level 0
    __syncwarp();
    while (sp > 0) {
        const int np = sp > kBatchBelow ? 1 : min(sp, kBatch);
        sp -= np;
        n_open += np;
        // lane L loads child slot L%8 of popped cells L/8 and 4 + L/8
        int ch[2] = {-1, -1}, lvs[2] = {0, 0};
        float4 pm[2], qa[2];
        float2 qb[2];
        float thr[2] = {0.0f, 0.0f};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            pm[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            qa[h] = pm[h];
            qb[h] = make_float2(0.0f, 0.0f);
            const int ci = cidx + 4 * h;
            if (ci < np) {
                const int e = stack[sp + ci];
                const int c = (e & kNodeMask) - n;
                lvs[h] = (int)((unsigned)e >> kNodeBits);
                ch[h] = __ldg(&s.wchild[c * 8 + slot]);
                if (ch[h] >= 0) {
                    pm[h] = __ldg(&s.wpm[c * 8 + slot]);
                    thr[h] = dq[lvs[h]];
                    if constexpr (kQuad) {
                        if (ch[h] >= n) {
                            qa[h] = __ldg(&s.wqa[c * 8 + slot]);
                            qb[h] = __ldg(&s.wqb[c * 8 + slot]);
                        }
                    }
                }
            }
        }
        // compact: bodies and cells in two dense lists, pop and slot order kept
        const bool isb0 = ch[0] >= 0 && ch[0] < n, isc0 = ch[0] >= n;
        const bool isb1 = ch[1] >= 0 && ch[1] < n, isc1 = ch[1] >= n;
        const unsigned mb0 = __ballot_sync(0xffffffffu, isb0), mc0 = __ballot_sync(0xffffffffu, isc0);
        const unsigned mb1 = __ballot_sync(0xffffffffu, isb1), mc1 = __ballot_sync(0xffffffffu, isc1);
        __syncwarp();  // the popped stack entries are read before pushes reuse them
        const int nb0 = __popc(mb0), nc0 = __popc(mc0);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const bool isb = h ? isb1 : isb0, isc = h ? isc1 : isc0;
            const unsigned mb = h ? mb1 : mb0, mc = h ? mc1 : mc0;
            if (isb) bpm[(h ? nb0 : 0) + __popc(mb & below)] = pm[h];
            if (isc) {
                const int k = (h ? nc0 : 0) + __popc(mc & below);
                cpm[k] = pm[h];
                cmeta[k] = make_float4(qb[h].x, qb[h].y, thr[h], __int_as_float(((lvs[h] + 1) << kNodeBits) | ch[h]));
                if constexpr (kQuad) cqa[k] = qa[h];
            }
        }
        __syncwarp();
        const int nb = nb0 + __popc(mb1), nc = nc0 + __popc(mc1);
        float bx = 0.0f, by = 0.0f, bz = 0.0f;  // batch sums (compensated mode)
        float &sx = kComp ? bx : ax, &sy = kComp ? by : ay, &sz = kComp ? bz : az;
        // child bodies: always accumulated
        n_body += nb;
#pragma unroll 4
        for (int k = 0; k < nb; ++k) {
            const float4 q = bpm[k];
            const float dx = q.x - P.x, dy = q.y - P.y, dz = q.z - P.z;
            const float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
            const float r = rsqrt_fast(d2);
            float F = q.w * (r * (r * r));
            if constexpr (kEpsZero) F = d2 > 0.0f ? F : 0.0f;
            sx = fmaf(dx, F, sx);
            sy = fmaf(dy, F, sy);
            sz = fmaf(dz, F, sz);
        }
        // child cells: accumulated when every lane accepts, else pushed; the
        // pushes of a round that cannot fill the stack skip the room test
        n_cell += nc;
        if (sp + nc <= kStack)
            cell_list<kQuad, false>(cpm, cmeta, cqa, nc, P, eps2, sx, sy, sz, stack, sp, n_drop, lane, ctrl);
        else
            cell_list<kQuad, true>(cpm, cmeta, cqa, nc, P, eps2, sx, sy, sz, stack, sp, n_drop, lane, ctrl);
        if constexpr (kComp) {  // one TwoSum per batch into the running sum
            two_sum_add(ax, lx, bx);
            two_sum_add(ay, ly, by);
            two_sum_add(az, lz, bz);
        }
        __syncwarp();
    }
    // every pushed cell is popped once, the root is popped without a push:
    // rejected cells = n_open - 1 + n_drop, accepted = staged - rejected
    n_cell -= n_open - 1u + n_drop;
    if (lane == 0) {
        const unsigned lanes = (unsigned)min(32, n - g * 32);
        atomicAdd(&ctrl->interactions, (unsigned long long)(n_body + n_cell) * lanes);
        atomicAdd(&ctrl->cell_interactions, (unsigned long long)n_cell * lanes);
        atomicAdd(&ctrl->opened, (unsigned long long)n_open);
    }
    if constexpr (kComp) {
        ax = ax + lx;
        ay = ay + ly;
        az = az + lz;
    }
    ax *= p.G;
    ay *= p.G;
    az *= p.G;
    if (valid) integrate_body<kMethod>(s, p, b, P, ax, ay, az);
}

}  // namespace nbgb
