// snapshot.cpp -- the snapshot file format of served and batched runs:
// positions, velocities and masses of one system at one step, float32
// little-endian, with a fixed 32-byte header.  Host code only (no device
// access), byte order written explicitly so files are the same on every
// host.
//
//   offset  size      field
//   0       8         magic "NBSNAP01"
//   8       4         uint32 format version (1)
//   12      4         uint32 N
//   16      8         int64  step
//   24      8         float64 simulated time
//   32      12 N      float32 positions  x0 y0 z0 x1 ...
//   32+12N  12 N      float32 velocities
//   32+24N  4 N       float32 masses
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/nbgb.h"

namespace {

constexpr char kMagic[8] = {'N', 'B', 'S', 'N', 'A', 'P', '0', '1'};
constexpr uint32_t kVersion = 1;

void put_u32(unsigned char *p, uint32_t v) {
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
void put_u64(unsigned char *p, uint64_t v) {
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get_u32(const unsigned char *p) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
    return v;
}
uint64_t get_u64(const unsigned char *p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
    return v;
}

bool write_floats(FILE *f, const float *a, size_t count) {
    std::vector<unsigned char> buf(4 * 4096);
    for (size_t i = 0; i < count; i += 4096) {
        const size_t m = count - i < 4096 ? count - i : 4096;
        for (size_t k = 0; k < m; ++k) {
            uint32_t u;
            memcpy(&u, &a[i + k], 4);
            put_u32(&buf[4 * k], u);
        }
        if (fwrite(buf.data(), 4, m, f) != m) return false;
    }
    return true;
}

bool read_floats(FILE *f, float *a, size_t count) {
    std::vector<unsigned char> buf(4 * 4096);
    for (size_t i = 0; i < count; i += 4096) {
        const size_t m = count - i < 4096 ? count - i : 4096;
        if (fread(buf.data(), 4, m, f) != m) return false;
        if (!a) continue;
        for (size_t k = 0; k < m; ++k) {
            const uint32_t u = get_u32(&buf[4 * k]);
            memcpy(&a[i + k], &u, 4);
        }
    }
    return true;
}

}  // namespace

extern "C" {

nb_status nb_snapshot_write(const char *path, int64_t step, double time, const float *pos3, const float *vel3,
                            const float *mass, int32_t n) {
    if (!path || !pos3 || !mass || n < 0) return NB_ERR_INVALID_ARGUMENT;
    FILE *f = fopen(path, "wb");
    if (!f) return NB_ERR_INVALID_ARGUMENT;
    unsigned char h[32];
    memcpy(h, kMagic, 8);
    put_u32(h + 8, kVersion);
    put_u32(h + 12, (uint32_t)n);
    put_u64(h + 16, (uint64_t)step);
    uint64_t tb;
    memcpy(&tb, &time, 8);
    put_u64(h + 24, tb);
    bool ok = fwrite(h, 1, 32, f) == 32 && write_floats(f, pos3, 3 * (size_t)n);
    if (ok) {
        if (vel3) {
            ok = write_floats(f, vel3, 3 * (size_t)n);
        } else {
            std::vector<float> zero(3 * (size_t)n, 0.0f);
            ok = write_floats(f, zero.data(), zero.size());
        }
    }
    ok = ok && write_floats(f, mass, (size_t)n);
    ok = (fclose(f) == 0) && ok;
    return ok ? NB_OK : NB_ERR_INVALID_ARGUMENT;
}

nb_status nb_snapshot_read(const char *path, int64_t *step, double *time, float *pos3, float *vel3, float *mass,
                           int32_t capacity, int32_t *n) {
    if (!path || !n) return NB_ERR_INVALID_ARGUMENT;
    FILE *f = fopen(path, "rb");
    if (!f) return NB_ERR_INVALID_ARGUMENT;
    unsigned char h[32];
    if (fread(h, 1, 32, f) != 32 || memcmp(h, kMagic, 8) != 0 || get_u32(h + 8) != kVersion) {
        fclose(f);
        return NB_ERR_INVALID_ARGUMENT;
    }
    const uint32_t count = get_u32(h + 12);
    *n = (int32_t)count;
    if (step) *step = (int64_t)get_u64(h + 16);
    if (time) {
        const uint64_t tb = get_u64(h + 24);
        memcpy(time, &tb, 8);
    }
    if (!pos3 && !vel3 && !mass) {  // header only
        fclose(f);
        return NB_OK;
    }
    if ((int64_t)count > (int64_t)capacity) {
        fclose(f);
        return NB_ERR_INVALID_ARGUMENT;
    }
    const bool ok = read_floats(f, pos3, 3 * (size_t)count) && read_floats(f, vel3, 3 * (size_t)count) &&
                    read_floats(f, mass, (size_t)count);
    fclose(f);
    return ok ? NB_OK : NB_ERR_INVALID_ARGUMENT;
}

nb_status nb_save_snapshot(nb_sim *sim, const char *path, int64_t step, double time) {
    if (!sim || !path) return NB_ERR_INVALID_ARGUMENT;
    nb_config c;
    nb_status st = nb_get_config(sim, &c);
    if (st != NB_OK) return st;
    const size_t n = (size_t)c.num_of_bodies;
    std::vector<float> pos(3 * n), vel(3 * n), mass(n);
    st = nb_get_state(sim, pos.data(), vel.data(), nullptr, mass.data());
    if (st != NB_OK) return st;
    return nb_snapshot_write(path, step, time, pos.data(), vel.data(), mass.data(), (int32_t)n);
}

}  // extern "C"
