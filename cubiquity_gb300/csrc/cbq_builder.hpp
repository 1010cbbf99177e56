// Canonical bulk DAG builder and the seeded synthetic scenes.
//
// The builder produces the same canonical sparse voxel DAG that the reference
// reaches through Volume::setVoxel followed by bake (src/library/storage.cpp:
// 396-437 and 208-290): every subtree whose voxels all hold one material is a
// material leaf (merge_node's collapse, storage.cpp:261-263) and identical
// subtrees are stored once.  Node indices differ from bake's hash-table
// placement; traversal depends only on the graph, which is identical.
//
// It works top-down over a Scene that can classify a power-of-two box as
// uniform or mixed, so the work is proportional to the surface, not the volume.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

namespace cbq {

constexpr uint32_t kMaterialCount = 256;   // storage.h:139
constexpr int kRootHeight = 32;            // raytracing.cpp:12

// A voxel scene confined to the box [origin, origin + 2^height)^3 (signed
// voxel coordinates; origin aligned to 2^height).
class Scene {
public:
    virtual ~Scene() = default;
    // Material of every voxel in [x, x+2^h) x [y, y+2^h) x [z, z+2^h) if they
    // all agree, else -1 ("mixed or unknown" is always a safe answer).
    virtual int classify(int32_t x, int32_t y, int32_t z, int h) const = 0;
    virtual uint8_t voxel(int32_t x, int32_t y, int32_t z) const = 0;
    int height = 0;
    int32_t origin[3] = {0, 0, 0};
};

// Flat node store in the reference layout: node i is words [8i, 8i+8), slots
// 0..255 are self-referencing material nodes (storage.cpp:110-122).
struct NodeArray {
    std::vector<uint32_t> words;
    uint32_t root = 0;
    uint64_t node_count() const { return words.size() / 8; }
};

// Hash-consing node table.
class NodeInterner {
public:
    NodeInterner();
    // Returns the index of the node with these children, creating it if new.
    // Eight equal material children collapse to that material.
    uint32_t intern(const uint32_t c[8]);
    std::vector<uint32_t>& words() { return words_; }
    const std::vector<uint32_t>& words() const { return words_; }
    uint64_t node_count() const { return words_.size() / 8; }

private:
    void grow();
    std::vector<uint32_t> words_;
    std::vector<uint32_t> table_;
    uint64_t mask_ = 0;
    uint64_t used_ = 0;
};

// Builds the canonical DAG of a scene on `threads` host threads (<= 0: all).
// The result is deterministic: it does not depend on the thread count.
NodeArray build_dag(const Scene& scene, int threads);

// Seeded scenes.
std::unique_ptr<Scene> make_sphere_scene(int edge_log2, int sphere_count, uint64_t seed);
std::unique_ptr<Scene> make_terrain_scene(int edge_log2, uint64_t seed);
std::unique_ptr<Scene> make_city_scene(int edge_log2, uint64_t seed);

}  // namespace cbq
