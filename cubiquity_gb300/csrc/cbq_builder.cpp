// Canonical bulk DAG builder and seeded scenes (see cbq_builder.hpp).
#include "cbq_builder.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

namespace cbq {

// ---------------------------------------------------------------------------
// Hash-consing
// ---------------------------------------------------------------------------

static inline uint64_t mix64(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

static inline uint64_t node_hash(const uint32_t* c)
{
    uint64_t a = (uint64_t)c[0] | ((uint64_t)c[1] << 32);
    uint64_t b = (uint64_t)c[2] | ((uint64_t)c[3] << 32);
    uint64_t d = (uint64_t)c[4] | ((uint64_t)c[5] << 32);
    uint64_t e = (uint64_t)c[6] | ((uint64_t)c[7] << 32);
    uint64_t h = mix64(a ^ 0x9e3779b97f4a7c15ull);
    h = mix64(h ^ b);
    h = mix64(h ^ d);
    h = mix64(h ^ e);
    return h;
}

static constexpr uint32_t kEmptySlot = 0xffffffffu;

NodeInterner::NodeInterner()
{
    words_.resize(8ull * kMaterialCount);
    for (uint32_t m = 0; m < kMaterialCount; m++)
        for (int k = 0; k < 8; k++) words_[8ull * m + k] = m;
    table_.assign(1024, kEmptySlot);
    mask_ = table_.size() - 1;
}

void NodeInterner::grow()
{
    std::vector<uint32_t> t(table_.size() * 2, kEmptySlot);
    const uint64_t mask = t.size() - 1;
    const uint64_t n = node_count();
    for (uint64_t i = kMaterialCount; i < n; i++) {
        uint64_t s = node_hash(&words_[8 * i]) & mask;
        while (t[s] != kEmptySlot) s = (s + 1) & mask;
        t[s] = (uint32_t)i;
    }
    table_.swap(t);
    mask_ = mask;
}

uint32_t NodeInterner::intern(const uint32_t c[8])
{
    if (c[0] < kMaterialCount) {
        bool uniform = true;
        for (int k = 1; k < 8; k++) uniform &= (c[k] == c[0]);
        if (uniform) return c[0];
    }
    uint64_t s = node_hash(c) & mask_;
    for (;;) {
        uint32_t idx = table_[s];
        if (idx == kEmptySlot) break;
        if (std::memcmp(&words_[8ull * idx], c, 32) == 0) return idx;
        s = (s + 1) & mask_;
    }
    const uint64_t idx = node_count();
    words_.insert(words_.end(), c, c + 8);
    table_[s] = (uint32_t)idx;
    if (++used_ * 2 > table_.size()) grow();
    return (uint32_t)idx;
}

// ---------------------------------------------------------------------------
// Builder
// ---------------------------------------------------------------------------

static uint32_t build_rec(const Scene& s, NodeInterner& in, int32_t x, int32_t y, int32_t z, int h)
{
    const int cls = s.classify(x, y, z, h);
    if (cls >= 0) return (uint32_t)cls;
    if (h == 0) return s.voxel(x, y, z);
    uint32_t c[8];
    const int32_t half = (int32_t)(1u << (h - 1));
    if (h == 1) {
        for (int i = 0; i < 8; i++)
            c[i] = s.voxel(x + ((i & 1) ? 1 : 0), y + ((i & 2) ? 1 : 0), z + ((i & 4) ? 1 : 0));
    } else {
        for (int i = 0; i < 8; i++)
            c[i] = build_rec(s, in, x + ((i & 1) ? half : 0), y + ((i & 2) ? half : 0),
                             z + ((i & 4) ? half : 0), h - 1);
    }
    return in.intern(c);
}

namespace {
struct Task {
    int32_t x, y, z;
    std::unique_ptr<NodeInterner> local;
    uint32_t local_root = 0;
};

uint32_t build_top(const Scene& s, NodeInterner& in, const std::vector<uint32_t>& task_roots, int split_h,
                   int tasks_per_axis, int32_t x, int32_t y, int32_t z, int h)
{
    if (h == split_h) {
        const int64_t tx = ((int64_t)x - s.origin[0]) >> split_h;
        const int64_t ty = ((int64_t)y - s.origin[1]) >> split_h;
        const int64_t tz = ((int64_t)z - s.origin[2]) >> split_h;
        return task_roots[(size_t)((tz * tasks_per_axis + ty) * tasks_per_axis + tx)];
    }
    const int cls = s.classify(x, y, z, h);
    if (cls >= 0) return (uint32_t)cls;
    uint32_t c[8];
    const int32_t half = (int32_t)(1u << (h - 1));
    for (int i = 0; i < 8; i++)
        c[i] = build_top(s, in, task_roots, split_h, tasks_per_axis, x + ((i & 1) ? half : 0),
                         y + ((i & 2) ? half : 0), z + ((i & 4) ? half : 0), h - 1);
    return in.intern(c);
}
}  // namespace

NodeArray build_dag(const Scene& scene, int threads)
{
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    const int H = scene.height;
    // Split the scene into independent subtrees of height split_h.
    int split_h = H;
    while (split_h > 6 && (1 << (3 * (H - split_h))) < 512) split_h--;
    const int per_axis = 1 << (H - split_h);
    std::vector<Task> tasks((size_t)per_axis * per_axis * per_axis);
    for (int tz = 0; tz < per_axis; tz++)
        for (int ty = 0; ty < per_axis; ty++)
            for (int tx = 0; tx < per_axis; tx++) {
                Task& t = tasks[(size_t)(tz * per_axis + ty) * per_axis + tx];
                t.x = scene.origin[0] + (tx << split_h);
                t.y = scene.origin[1] + (ty << split_h);
                t.z = scene.origin[2] + (tz << split_h);
            }
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (;;) {
            size_t i = next.fetch_add(1);
            if (i >= tasks.size()) break;
            Task& t = tasks[i];
            t.local = std::make_unique<NodeInterner>();
            t.local_root = build_rec(scene, *t.local, t.x, t.y, t.z, split_h);
        }
    };
    {
        std::vector<std::thread> pool;
        const int nt = std::min<int>(threads, (int)tasks.size());
        for (int i = 1; i < nt; i++) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
    }

    // Merge the per-task node sets in task order (deterministic indices).
    NodeInterner global;
    std::vector<uint32_t> task_roots(tasks.size());
    std::vector<uint32_t> remap;
    for (size_t i = 0; i < tasks.size(); i++) {
        Task& t = tasks[i];
        const std::vector<uint32_t>& w = t.local->words();
        const uint64_t n = w.size() / 8;
        remap.assign(n, 0);
        for (uint64_t m = 0; m < kMaterialCount; m++) remap[m] = (uint32_t)m;
        for (uint64_t k = kMaterialCount; k < n; k++) {
            uint32_t c[8];
            for (int j = 0; j < 8; j++) c[j] = remap[w[8 * k + j]];
            remap[k] = global.intern(c);
        }
        task_roots[i] = remap[t.local_root];
        t.local.reset();
    }
    uint32_t node = build_top(scene, global, task_roots, split_h, per_axis, scene.origin[0], scene.origin[1],
                              scene.origin[2], H);

    // Chain of single-child nodes from the scene box up to the root at height 32.
    // Child ids come from the unsigned positions (signed + 2^31, storage.cpp:45-67).
    const uint32_t ux = (uint32_t)scene.origin[0] + 0x80000000u;
    const uint32_t uy = (uint32_t)scene.origin[1] + 0x80000000u;
    const uint32_t uz = (uint32_t)scene.origin[2] + 0x80000000u;
    for (int hh = H + 1; hh <= kRootHeight; hh++) {
        const int bit = hh - 1;
        const uint32_t cid = ((ux >> bit) & 1u) | (((uy >> bit) & 1u) << 1) | (((uz >> bit) & 1u) << 2);
        uint32_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        c[cid] = node;
        node = global.intern(c);
    }
    NodeArray out;
    out.words = std::move(global.words());
    out.root = node;
    return out;
}

// ---------------------------------------------------------------------------
// Deterministic random numbers (identical on every platform)
// ---------------------------------------------------------------------------

static inline uint64_t splitmix64(uint64_t& state)
{
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static inline uint64_t hash_u64(uint64_t a, uint64_t b, uint64_t c, uint64_t d)
{
    uint64_t s = a * 0x9e3779b97f4a7c15ull ^ mix64(b + 0x632be59bd9b4e019ull);
    s = mix64(s ^ (c * 0xd6e8feb86659fd93ull));
    s = mix64(s ^ (d * 0xa0761d6478bd642full));
    return s;
}

// Uniform integer in [lo, hi].
static inline int64_t uniform_int(uint64_t& st, int64_t lo, int64_t hi)
{
    const uint64_t range = (uint64_t)(hi - lo + 1);
    return lo + (int64_t)(((unsigned __int128)splitmix64(st) * range) >> 64);
}

// Uniform double in [0, 1) from the top 53 bits.
static inline double unit_double(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

static inline double fade(double t) { return t * t * (3.0 - 2.0 * t); }

// ---------------------------------------------------------------------------
// Sphere scene: N spheres, centres uniform in [E/8, 7E/8]^3, radii uniform in
// [E/32, 5E/32], material 1 + (i mod 7), first sphere wins; then a ground slab
// z < E/8 of material 8.  For E = 256: centres in [32,224], radii 8..40, slab z<32.
// ---------------------------------------------------------------------------

namespace {

class SphereScene final : public Scene {
public:
    SphereScene(int edge_log2, int count, uint64_t seed)
    {
        height = edge_log2;
        edge_ = 1 << edge_log2;
        uint64_t st = seed;
        const int64_t lo = edge_ / 8, hi = 7 * (int64_t)edge_ / 8;
        const int64_t rlo = std::max<int64_t>(1, edge_ / 32), rhi = std::max<int64_t>(1, 5 * (int64_t)edge_ / 32);
        for (int i = 0; i < count; i++) {
            Sphere s;
            s.cx = uniform_int(st, lo, hi);
            s.cy = uniform_int(st, lo, hi);
            s.cz = uniform_int(st, lo, hi);
            s.r = uniform_int(st, rlo, rhi);
            s.mat = (uint8_t)(1 + (i % 7));
            spheres_.push_back(s);
        }
        slab_ = edge_ / 8;
    }

    uint8_t voxel(int32_t x, int32_t y, int32_t z) const override
    {
        if (x < 0 || y < 0 || z < 0 || x >= edge_ || y >= edge_ || z >= edge_) return 0;
        for (const Sphere& s : spheres_) {
            const int64_t dx = x - s.cx, dy = y - s.cy, dz = z - s.cz;
            if (dx * dx + dy * dy + dz * dz <= s.r * s.r) return s.mat;
        }
        return z < slab_ ? 8 : 0;
    }

    int classify(int32_t x, int32_t y, int32_t z, int h) const override
    {
        const int64_t s1 = ((int64_t)1 << h) - 1;  // last voxel offset
        for (const Sphere& s : spheres_) {
            int64_t dmin = 0, dmax = 0;
            const int64_t lo[3] = {x, y, z};
            const int64_t c[3] = {s.cx, s.cy, s.cz};
            for (int a = 0; a < 3; a++) {
                const int64_t l = lo[a], u = lo[a] + s1;
                const int64_t near = std::clamp(c[a], l, u);
                const int64_t dn = c[a] - near;
                const int64_t df = std::max(std::abs(c[a] - l), std::abs(c[a] - u));
                dmin += dn * dn;
                dmax += df * df;
            }
            const int64_t r2 = s.r * s.r;
            if (dmin > r2) continue;            // sphere misses the box
            if (dmax <= r2) return s.mat;       // first touching sphere covers it
            return -1;
        }
        if ((int64_t)z + s1 < slab_) return 8;
        if (z >= slab_) return 0;
        return -1;
    }

private:
    struct Sphere {
        int64_t cx, cy, cz, r;
        uint8_t mat;
    };
    std::vector<Sphere> spheres_;
    int32_t edge_ = 0;
    int32_t slab_ = 0;
};

// ---------------------------------------------------------------------------
// Terrain scene (edge E): column heights from 6-octave fBm value noise (base
// period E/4, gain 0.5, lacunarity 2) mapped to [E/8, E/2]; caves where 3D value
// noise (period E/32, lattice values uniform in [-1,1)) exceeds 0.35; material
// 1 + ((z / (E/32)) mod 16), i.e. 16 bands by height.  E = 4096: period 1024,
// heights in [512, 2048], cave period 128, bands of 128 voxels.
// ---------------------------------------------------------------------------

class TerrainScene final : public Scene {
public:
    TerrainScene(int edge_log2, uint64_t seed) : seed_(seed)
    {
        height = edge_log2;
        edge_ = 1 << edge_log2;
        hmin_ = edge_ / 8;
        hmax_ = edge_ / 2;
        band_log2_ = std::max(0, edge_log2 - 5);
        cave_log2_ = std::max(0, edge_log2 - 5);
        base_log2_ = edge_log2 - 2;
        make_heights();
        make_cave_lattice();
    }

    uint8_t voxel(int32_t x, int32_t y, int32_t z) const override
    {
        if (x < 0 || y < 0 || z < 0 || x >= edge_ || y >= edge_ || z >= edge_) return 0;
        if (z >= (int32_t)heights_[(size_t)y * edge_ + x]) return 0;
        if (cave_noise(x, y, z) > kCaveThreshold) return 0;
        return material(z);
    }

    int classify(int32_t x, int32_t y, int32_t z, int h) const override
    {
        const int level = h;
        const size_t w = (size_t)edge_ >> level;
        const size_t idx = (size_t)(y >> level) * w + (size_t)(x >> level);
        const int32_t top = (int32_t)mip_max_[level][idx];
        const int32_t bottom = (int32_t)mip_min_[level][idx];
        const int32_t s = 1 << h;
        if (z >= top) return 0;
        if (h <= 1) return -1;
        double cmin, cmax;
        cave_bounds(x, y, z, h, cmin, cmax);
        if (cmin > kCaveThreshold + kEps) return 0;
        if (z + s <= bottom && cmax < kCaveThreshold - kEps && h <= band_log2_) return material(z);
        return -1;
    }

private:
    static constexpr double kCaveThreshold = 0.35;
    static constexpr double kEps = 1e-9;

    uint8_t material(int32_t z) const { return (uint8_t)(1 + ((z >> band_log2_) & 15)); }

    double lattice2(int octave, int64_t i, int64_t j) const
    {
        return unit_double(hash_u64(seed_, 0x100 + octave, (uint64_t)i, (uint64_t)j));
    }

    void make_heights()
    {
        heights_.assign((size_t)edge_ * edge_, 0);
        const int octaves = 6;
        // Precomputed lattice per octave.
        std::vector<std::vector<double>> lat(octaves);
        std::vector<int> per(octaves), cells(octaves);
        for (int o = 0; o < octaves; o++) {
            per[o] = 1 << std::max(0, base_log2_ - o);  // octaves finer than a voxel repeat the voxel
            cells[o] = edge_ / per[o] + 1;
            lat[o].resize((size_t)cells[o] * cells[o]);
            for (int j = 0; j < cells[o]; j++)
                for (int i = 0; i < cells[o]; i++) lat[o][(size_t)j * cells[o] + i] = lattice2(o, i, j);
        }
        const double norm = 1.0 + 0.5 + 0.25 + 0.125 + 0.0625 + 0.03125;
        const int nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
        std::atomic<int> next{0};
        auto work = [&]() {
            for (;;) {
                const int y = next.fetch_add(1);
                if (y >= edge_) break;
                for (int x = 0; x < edge_; x++) {
                    double sum = 0.0, amp = 1.0;
                    for (int o = 0; o < octaves; o++) {
                        const int p = per[o];
                        const int ci = x / p, cj = y / p;
                        const double tx = fade((double)(x - ci * p) / p), ty = fade((double)(y - cj * p) / p);
                        const double* L = lat[o].data();
                        const int C = cells[o];
                        const double v00 = L[(size_t)cj * C + ci], v10 = L[(size_t)cj * C + ci + 1];
                        const double v01 = L[(size_t)(cj + 1) * C + ci], v11 = L[(size_t)(cj + 1) * C + ci + 1];
                        const double a = v00 + (v10 - v00) * tx;
                        const double b = v01 + (v11 - v01) * tx;
                        sum += amp * (a + (b - a) * ty);
                        amp *= 0.5;
                    }
                    const double v = sum / norm;
                    int32_t hgt = hmin_ + (int32_t)std::floor((double)(hmax_ - hmin_) * v);
                    hgt = std::clamp(hgt, hmin_, hmax_);
                    heights_[(size_t)y * edge_ + x] = (uint16_t)hgt;
                }
            }
        };
        std::vector<std::thread> pool;
        for (int i = 1; i < nthreads; i++) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
        // Min/max pyramids over aligned 2^k x 2^k footprints.
        const int levels = height + 1;
        mip_min_.resize(levels);
        mip_max_.resize(levels);
        mip_min_[0] = heights_;
        mip_max_[0] = heights_;
        for (int l = 1; l < levels; l++) {
            const size_t w = (size_t)edge_ >> l, pw = (size_t)edge_ >> (l - 1);
            mip_min_[l].resize(w * w);
            mip_max_[l].resize(w * w);
            for (size_t j = 0; j < w; j++)
                for (size_t i = 0; i < w; i++) {
                    const size_t a = (2 * j) * pw + 2 * i, b = a + 1, c = a + pw, d = c + 1;
                    mip_min_[l][j * w + i] = std::min({mip_min_[l - 1][a], mip_min_[l - 1][b],
                                                       mip_min_[l - 1][c], mip_min_[l - 1][d]});
                    mip_max_[l][j * w + i] = std::max({mip_max_[l - 1][a], mip_max_[l - 1][b],
                                                       mip_max_[l - 1][c], mip_max_[l - 1][d]});
                }
        }
    }

    void make_cave_lattice()
    {
        cave_cells_ = (edge_ >> cave_log2_) + 1;
        const size_t n = (size_t)cave_cells_ * cave_cells_ * cave_cells_;
        cave_lat_.resize(n);
        for (int k = 0; k < cave_cells_; k++)
            for (int j = 0; j < cave_cells_; j++)
                for (int i = 0; i < cave_cells_; i++)
                    cave_lat_[((size_t)k * cave_cells_ + j) * cave_cells_ + i] =
                        2.0 * unit_double(hash_u64(seed_, 0x200, (uint64_t)i, ((uint64_t)j << 32) | (uint64_t)k)) - 1.0;
    }

    double cave_lat(int i, int j, int k) const
    {
        return cave_lat_[((size_t)k * cave_cells_ + j) * cave_cells_ + i];
    }

    double cave_noise(int32_t x, int32_t y, int32_t z) const
    {
        const int ci = x >> cave_log2_, cj = y >> cave_log2_, ck = z >> cave_log2_;
        const double p = (double)(1 << cave_log2_);
        const double tx = fade((double)(x - (ci << cave_log2_)) / p);
        const double ty = fade((double)(y - (cj << cave_log2_)) / p);
        const double tz = fade((double)(z - (ck << cave_log2_)) / p);
        const double c000 = cave_lat(ci, cj, ck), c100 = cave_lat(ci + 1, cj, ck);
        const double c010 = cave_lat(ci, cj + 1, ck), c110 = cave_lat(ci + 1, cj + 1, ck);
        const double c001 = cave_lat(ci, cj, ck + 1), c101 = cave_lat(ci + 1, cj, ck + 1);
        const double c011 = cave_lat(ci, cj + 1, ck + 1), c111 = cave_lat(ci + 1, cj + 1, ck + 1);
        const double x00 = c000 + (c100 - c000) * tx, x10 = c010 + (c110 - c010) * tx;
        const double x01 = c001 + (c101 - c001) * tx, x11 = c011 + (c111 - c011) * tx;
        const double y0 = x00 + (x10 - x00) * ty, y1 = x01 + (x11 - x01) * ty;
        return y0 + (y1 - y0) * tz;
    }

    // Bounds of the cave noise over the voxels of the box.  Inside one lattice
    // cell the noise is multilinear in the (monotone) faded coordinates, so its
    // extremes over a box sit at the box corners; across cells it is a convex
    // combination of the lattice values it touches.
    void cave_bounds(int32_t x, int32_t y, int32_t z, int h, double& lo, double& hi) const
    {
        if (h <= cave_log2_) {
            const int32_t s1 = (1 << h) - 1;
            lo = 1e300;
            hi = -1e300;
            for (int c = 0; c < 8; c++) {
                const double v = cave_noise(x + ((c & 1) ? s1 : 0), y + ((c & 2) ? s1 : 0), z + ((c & 4) ? s1 : 0));
                lo = std::min(lo, v);
                hi = std::max(hi, v);
            }
            return;
        }
        const int i0 = x >> cave_log2_, j0 = y >> cave_log2_, k0 = z >> cave_log2_;
        const int n = 1 << (h - cave_log2_);
        lo = 1e300;
        hi = -1e300;
        for (int k = k0; k <= k0 + n && k < cave_cells_; k++)
            for (int j = j0; j <= j0 + n && j < cave_cells_; j++)
                for (int i = i0; i <= i0 + n && i < cave_cells_; i++) {
                    const double v = cave_lat(i, j, k);
                    lo = std::min(lo, v);
                    hi = std::max(hi, v);
                }
    }

    uint64_t seed_;
    int32_t edge_ = 0, hmin_ = 0, hmax_ = 0;
    int band_log2_ = 0, cave_log2_ = 0, base_log2_ = 0;
    std::vector<uint16_t> heights_;
    std::vector<std::vector<uint16_t>> mip_min_, mip_max_;
    int cave_cells_ = 0;
    std::vector<double> cave_lat_;
};

// ---------------------------------------------------------------------------
// City scene (edge E): axis-aligned boxes on a 64-voxel grid.  Each grid cell
// holds at most one building with a footprint of 16..56 voxels per side and a
// height log-uniform in [32, 2048] (clamped to E/2), one of 32 materials; a
// ground slab z < 16 of material 1.
// ---------------------------------------------------------------------------

class CityScene final : public Scene {
public:
    CityScene(int edge_log2, uint64_t seed) : seed_(seed)
    {
        height = edge_log2;
        edge_ = 1 << edge_log2;
        cells_ = edge_ / kGrid;
        blds_.resize((size_t)cells_ * cells_);
        uint64_t st = seed;
        const double lmin = std::log(32.0), lmax = std::log((double)std::min(2048, edge_ / 2));
        for (int j = 0; j < cells_; j++)
            for (int i = 0; i < cells_; i++) {
                Building& b = blds_[(size_t)j * cells_ + i];
                const int64_t wx = uniform_int(st, 16, 56), wy = uniform_int(st, 16, 56);
                const int64_t ox = uniform_int(st, 0, kGrid - wx), oy = uniform_int(st, 0, kGrid - wy);
                const double u = unit_double(splitmix64(st));
                const int64_t hh = (int64_t)std::floor(std::exp(lmin + (lmax - lmin) * u));
                b.x0 = i * kGrid + (int32_t)ox;
                b.y0 = j * kGrid + (int32_t)oy;
                b.x1 = b.x0 + (int32_t)wx;
                b.y1 = b.y0 + (int32_t)wy;
                b.top = kGround + (int32_t)hh;
                b.mat = (uint8_t)(2 + uniform_int(st, 0, 31));
            }
    }

    uint8_t voxel(int32_t x, int32_t y, int32_t z) const override
    {
        if (x < 0 || y < 0 || z < 0 || x >= edge_ || y >= edge_ || z >= edge_) return 0;
        if (z < kGround) return 1;
        const Building& b = blds_[(size_t)(y / kGrid) * cells_ + (x / kGrid)];
        if (x >= b.x0 && x < b.x1 && y >= b.y0 && y < b.y1 && z < b.top) return b.mat;
        return 0;
    }

    int classify(int32_t x, int32_t y, int32_t z, int h) const override
    {
        const int64_t s = (int64_t)1 << h;
        const int64_t x1 = x + s, y1 = y + s, z1 = z + s;
        if (z1 <= kGround) return 1;
        if (z < kGround) return -1;
        // Buildings touching the box footprint.
        const int ci0 = x / kGrid, cj0 = y / kGrid;
        const int ci1 = (int)((x1 - 1) / kGrid), cj1 = (int)((y1 - 1) / kGrid);
        int found = -1;
        int64_t touched = 0;
        for (int j = cj0; j <= cj1; j++)
            for (int i = ci0; i <= ci1; i++) {
                const Building& b = blds_[(size_t)j * cells_ + i];
                if (b.x1 <= x || b.x0 >= x1 || b.y1 <= y || b.y0 >= y1 || b.top <= z) continue;
                touched++;
                const bool covers = b.x0 <= x && b.x1 >= x1 && b.y0 <= y && b.y1 >= y1 && b.top >= z1;
                if (covers && touched == 1) found = b.mat;
                else return -1;
            }
        if (touched == 0) return 0;
        return found;
    }

private:
    static constexpr int32_t kGrid = 64;
    static constexpr int32_t kGround = 16;
    struct Building {
        int32_t x0, y0, x1, y1, top;
        uint8_t mat;
    };
    uint64_t seed_;
    int32_t edge_ = 0;
    int cells_ = 0;
    std::vector<Building> blds_;
};

}  // namespace

std::unique_ptr<Scene> make_sphere_scene(int edge_log2, int sphere_count, uint64_t seed)
{
    return std::make_unique<SphereScene>(edge_log2, sphere_count, seed);
}

std::unique_ptr<Scene> make_terrain_scene(int edge_log2, uint64_t seed)
{
    return std::make_unique<TerrainScene>(edge_log2, seed);
}

std::unique_ptr<Scene> make_city_scene(int edge_log2, uint64_t seed)
{
    return std::make_unique<CityScene>(edge_log2, seed);
}

}  // namespace cbq
