// Synthetic scenes for the benchmark and the tests (no reference
// counterpart: the reference generates chunks with 3-D OpenSimplex noise,
// chunk.rs:56-109).  Everything here is integer hashing plus IEEE double
// arithmetic compiled without FMA contraction, so it yields the same blocks
// and cameras on every host.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/vrg.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
inline uint64_t hash4(uint64_t seed, int64_t a, int64_t b, int64_t c) {
    uint64_t h = splitmix64(seed);
    h = splitmix64(h ^ (uint64_t)a);
    h = splitmix64(h ^ (uint64_t)b * 0x632BE59BD9B4E019ull);
    h = splitmix64(h ^ (uint64_t)c * 0x85157AF5ull);
    return h;
}
inline double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

// value noise: hashed lattice values, smoothstep-weighted bilinear blend
double value_noise(uint64_t seed, double x, double z) {
    double fx = std::floor(x), fz = std::floor(z);
    int64_t ix = (int64_t)fx, iz = (int64_t)fz;
    double tx = x - fx, tz = z - fz;
    double sx = tx * tx * (3.0 - 2.0 * tx), sz = tz * tz * (3.0 - 2.0 * tz);
    double v00 = unit(hash4(seed, ix, iz, 0)), v10 = unit(hash4(seed, ix + 1, iz, 0));
    double v01 = unit(hash4(seed, ix, iz + 1, 0)), v11 = unit(hash4(seed, ix + 1, iz + 1, 0));
    double a = v00 + (v10 - v00) * sx;
    double b = v01 + (v11 - v01) * sx;
    return a + (b - a) * sz;
}

int column_height(uint64_t seed, int64_t x, int64_t z) {
    // 2 octaves: period 16 blocks, then period 8 at half amplitude
    double h = value_noise(seed, (double)x / 16.0, (double)z / 16.0) +
               0.5 * value_noise(seed ^ 0x5bd1e995ull, (double)x / 8.0, (double)z / 8.0);
    h = h / 1.5;  // [0, 1)
    int height = 8 + (int)std::floor(h * 17.0);
    if (height < 8) height = 8;
    if (height > 24) height = 24;
    return height;  // blocks y < height are solid
}

}  // namespace

extern "C" {

VRG_API vrg_status vrg_terrain_materials(uint64_t seed, vrg_material *mats, uint32_t cap, uint32_t *n) {
    const uint32_t types = 6 + 16;
    if (!mats || !n || cap < 6 * types) return VRG_ERR_INVALID_ARGUMENT;
    memset(mats, 0, 6 * types * sizeof(vrg_material));
    for (uint32_t t = 0; t < types; t++) {
        uint64_t h = hash4(seed, 0x6d617400, t, 0);
        float alb[3], em[3] = {0.0f, 0.0f, 0.0f};
        for (int c = 0; c < 3; c++) alb[c] = (float)(0.2 + 0.6 * unit(hash4(h, c, 1, 0)));
        if (t >= 6)
            for (int c = 0; c < 3; c++) em[c] = (float)(5.0 + 15.0 * unit(hash4(h, c, 2, 0)));
        for (int f = 0; f < 6; f++) {
            vrg_material &m = mats[6 * t + f];
            for (int c = 0; c < 3; c++) {
                m.reflectivity[c] = alb[c];
                m.emission[c] = em[c];
            }
            m.alpha = 1.0f;
            m.metallic = 0.0f;
            // texture luminance of a uniform emissivity texture whose texel is
            // emission/1000 in [0,1]: mean(r8+g8+b8) = 255*(r+g+b)/1000
            m.luminance = (em[0] + em[1] + em[2]) * 0.255f;
            m.flags = 0;
        }
    }
    *n = 6 * types;
    return VRG_OK;
}

VRG_API vrg_status vrg_terrain_generate(uint64_t seed, uint32_t nx, uint32_t nz, float emissive, uint8_t *blocks) {
    if (!blocks || nx == 0 || nz == 0 || nx > 256 || nz > 256) return VRG_ERR_INVALID_ARGUMENT;
    const uint8_t AIR = 22;  // 6 Lambertian + 16 emissive block types
    const int64_t X = 32 * (int64_t)nx, Z = 32 * (int64_t)nz;
    auto idx = [&](int64_t x, int64_t y, int64_t z) -> size_t {
        int64_t cx = x >> 5, cz = z >> 5;
        return (size_t)(cx * nz + cz) * VRG_CHUNK_BLOCKS + (size_t)((x & 31) * 1024 + y * 32 + (z & 31));
    };
    std::vector<int> hgt((size_t)(X * Z));
    for (int64_t x = 0; x < X; x++)
        for (int64_t z = 0; z < Z; z++) hgt[(size_t)(x * Z + z)] = column_height(seed, x, z);
    auto H = [&](int64_t x, int64_t z) -> int {
        if (x < 0 || z < 0 || x >= X || z >= Z) return 0;  // outside the world: air
        return hgt[(size_t)(x * Z + z)];
    };
    if (!(emissive >= 0.0f)) return VRG_ERR_INVALID_ARGUMENT;
    const uint64_t thr = emissive >= 1.0f ? UINT64_MAX : (uint64_t)((double)emissive * 18446744073709551616.0);
    for (int64_t x = 0; x < X; x++)
        for (int64_t z = 0; z < Z; z++) {
            int h = H(x, z);
            int hmin = h;  // lowest neighbouring column: blocks at y >= hmin - ... are exposed
            int nbh[4] = {H(x - 1, z), H(x + 1, z), H(x, z - 1), H(x, z + 1)};
            for (int k = 0; k < 4; k++) hmin = nbh[k] < hmin ? nbh[k] : hmin;
            for (int64_t y = 0; y < 32; y++) {
                uint8_t b = AIR;
                if (y < h) {
                    b = (uint8_t)(hash4(seed ^ 0xb10c5ull, x, y, z) % 6);
                    // surface block: top of the column or exposed on a side
                    // (the bottom layer rests on solid ground)
                    bool surface = (y == h - 1) || (y >= hmin);
                    if (surface && hash4(seed ^ 0x11647ull, x, y, z) < thr)
                        b = (uint8_t)(6 + hash4(seed ^ 0xe3155ull, x, y, z) % 16);
                }
                blocks[idx(x, y, z)] = b;
            }
        }
    return VRG_OK;
}

VRG_API vrg_status vrg_orbit_camera(uint32_t nx, uint32_t nz, uint32_t frame, uint32_t n_frames, uint32_t width,
                                    uint32_t height, vrg_camera *cam) {
    if (!cam || n_frames == 0 || width == 0 || height == 0) return VRG_ERR_INVALID_ARGUMENT;
    const double cx = 16.0 * nx, cz = 16.0 * nz, cy = 14.0;
    const double ext = 16.0 * (nx > nz ? nx : nz);
    const double R = ext * 1.1 + 20.0, Y = cy + ext * 0.6 + 16.0;
    const double th = 2.0 * 3.14159265358979323846 * (double)frame / (double)n_frames + 0.6;
    double eye[3] = {cx + R * std::cos(th), Y, cz + R * std::sin(th)};
    double f[3] = {cx - eye[0], cy - eye[1], cz - eye[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double &v : f) v /= fl;
    // right = front x worldup, up = right x front, worldup = (0,-1,0) (camera.rs:22-35,100)
    const double wu[3] = {0.0, -1.0, 0.0};
    double r[3] = {f[1] * wu[2] - f[2] * wu[1], f[2] * wu[0] - f[0] * wu[2], f[0] * wu[1] - f[1] * wu[0]};
    double rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (double &v : r) v /= rl;
    double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (double &v : u) v /= ul;
    // half field of view: tan = 0.55 vertically
    for (int i = 0; i < 3; i++) {
        cam->eye[i] = (float)eye[i];
        cam->front[i] = (float)f[i];
        cam->right[i] = (float)(r[i] * 0.55);
        cam->up[i] = (float)(u[i] * 0.55);
    }
    cam->width = width;
    cam->height = height;
    return VRG_OK;
}

// PCG32 (O'Neill 2014): 64-bit LCG state, xorshift-high + random rotation output.
VRG_API uint32_t vrg_pcg32_next(uint64_t *state, uint64_t inc) {
    uint64_t old = *state;
    *state = old * 6364136223846793005ull + (inc | 1ull);
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

}  // extern "C"
