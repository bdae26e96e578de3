// Blue-noise tile generator: void-and-cluster (Ulichney, "The void-and-
// cluster method for dither array generation", SPIE 1993), toroidal
// Gaussian energy with sigma 1.5, one independent rank map per RGBA
// channel, ranks spread uniformly over 0..255.
//
// The reference ships a 256x256 RGBA8 blue-noise PNG decoded with lodepng
// (renderer.ixx:101-110) and samples it with texelFetch at Gid % size
// (secondaryRays.comp:125).  The workloads here use a 64x64 tile generated
// from a seed instead, so nothing has to be shipped; any RGBA8 tile, the
// reference's included, can be passed to mrt_cuda_blue_noise_upload.
#include "mrt_host.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct VoidCluster {
    int n, N;
    std::vector<double> lut;    // toroidal Gaussian, indexed by (dy*n + dx)
    std::vector<double> energy; // sum over set pixels of lut(distance)
    std::vector<uint8_t> bits;

    explicit VoidCluster(int size) : n(size), N(size * size), lut(N), energy(N, 0.0), bits(N, 0) {
        const double sigma = 1.5;
        for (int dy = 0; dy < n; ++dy)
            for (int dx = 0; dx < n; ++dx) {
                int ddx = std::min(dx, n - dx), ddy = std::min(dy, n - dy);
                lut[dy * n + dx] = std::exp(-(ddx * ddx + ddy * ddy) / (2.0 * sigma * sigma));
            }
    }
    void flip(int p, bool on) {
        bits[p] = on;
        int py = p / n, px = p % n;
        double s = on ? 1.0 : -1.0;
        for (int y = 0; y < n; ++y) {
            int dy = (y - py + n) % n;
            for (int x = 0; x < n; ++x) {
                int dx = (x - px + n) % n;
                energy[y * n + x] += s * lut[dy * n + dx];
            }
        }
    }
    // tightest cluster among pixels with bits == v (max energy), or largest
    // void among pixels with bits == v (min energy); ties -> lowest index
    int extreme(uint8_t v, bool want_max) const {
        int best = -1;
        for (int i = 0; i < N; ++i) {
            if (bits[i] != v) continue;
            if (best < 0 || (want_max ? energy[i] > energy[best] : energy[i] < energy[best])) best = i;
        }
        return best;
    }
    void rebuild() {
        std::fill(energy.begin(), energy.end(), 0.0);
        std::vector<uint8_t> b = bits;
        std::fill(bits.begin(), bits.end(), 0);
        for (int i = 0; i < N; ++i)
            if (b[i]) flip(i, true);
    }
};

void rank_map(int n, uint64_t seed, std::vector<int>& rank) {
    VoidCluster vc(n);
    const int N = n * n;
    uint64_t s = seed;
    // initial binary pattern: ~10% minority pixels
    int ones = std::max(1, N / 10);
    int placed = 0;
    while (placed < ones) {
        int p = int(splitmix(s) % uint64_t(N));
        if (!vc.bits[p]) { vc.flip(p, true); placed++; }
    }
    // relax: move the tightest cluster into the largest void until stable
    for (int it = 0; it < 4 * N; ++it) {
        int c = vc.extreme(1, true);
        vc.flip(c, false);
        int v = vc.extreme(0, false);
        vc.flip(v, true);
        if (v == c) break;
    }
    std::vector<uint8_t> proto = vc.bits;
    rank.assign(N, -1);
    // phase 1: rank the prototype's ones by removing tightest clusters
    {
        int r = ones - 1;
        while (r >= 0) {
            int c = vc.extreme(1, true);
            vc.flip(c, false);
            rank[c] = r--;
        }
    }
    // phase 2: from the prototype, fill the largest voids up to half
    vc.bits = proto;
    vc.rebuild();
    int r = ones;
    while (r < N / 2) {
        int v = vc.extreme(0, false);
        vc.flip(v, true);
        rank[v] = r++;
    }
    // phase 3: the remaining zeros are the minority; rank by tightest
    // cluster of zeros = the zero pixel with the highest energy of zeros,
    // i.e. the lowest energy of ones
    while (r < N) {
        int v = vc.extreme(0, false);
        vc.flip(v, true);
        rank[v] = r++;
    }
}

} // namespace

extern "C" int mrt_blue_noise_generate(uint32_t seed, uint32_t size, uint8_t* rgba_out) {
    if (!rgba_out || size < 4 || size > 256) return MRT_EINVAL;
    const int n = int(size), N = n * n;
    std::vector<int> rank;
    for (int ch = 0; ch < 4; ++ch) {
        rank_map(n, (uint64_t(seed) << 8) ^ uint64_t(0xB10E + 977 * ch), rank);
        for (int i = 0; i < N; ++i) rgba_out[4 * i + ch] = uint8_t((int64_t(rank[i]) * 256) / N);
    }
    return MRT_OK;
}
