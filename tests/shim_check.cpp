// Drives the C++ drop-in shim (include/cubiquity_gb300.hpp) the way the
// reference's callers drive Cubiquity::intersectVolume: load a .dag, upload it,
// compute its SubDAGs, cast rays one at a time (both overloads) and in a batch,
// check that foreign SubDAGs are refused, and write the 48-byte
// RayVolumeIntersection records to a file for the test to compare.
//
//   shim_check <volume.dag> <rays.bin: n x 6 float32> <out.bin>
#include "cubiquity_gb300.hpp"

#include <cstdio>
#include <vector>

int main(int argc, char** argv)
{
    if (argc != 4) {
        std::fprintf(stderr, "usage: shim_check volume.dag rays.bin out.bin\n");
        return 2;
    }
    uint32_t* nodes = nullptr;
    uint64_t count = 0;
    uint32_t root = 0;
    cbq::check(cbq_dag_load(argv[1], &nodes, &count, &root), "load");
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    std::vector<float> rays;
    float buf[6];
    while (std::fread(buf, sizeof(float), 6, f) == 6) rays.insert(rays.end(), buf, buf + 6);
    std::fclose(f);
    const size_t n = rays.size() / 6;
    try {
        cbq::Volume vol(nodes, count, root);
        std::vector<cbq::RayVolumeIntersection> out(n);
        // First half one ray at a time (collision-query style), through the two
        // overloads in turn (six floats, Ray3f); second half batched.
        const cbq::SubDAGArray subDAGs = cbq::findSubDAGs(nodes, count, root);
        const size_t half = n / 2;
        for (size_t i = 0; i < half; i++) {
            const float* r = &rays[6 * i];
            if (i % 2 == 0) {
                out[i] = cbq::intersectVolume(vol, subDAGs, r[0], r[1], r[2], r[3], r[4], r[5], true);
            } else {
                const cbq::Ray3f ray(cbq::vec3{r[0], r[1], r[2]}, cbq::vec3{r[3], r[4], r[5]});
                out[i] = cbq::intersectVolume(vol, subDAGs, ray, true);
            }
        }
        // SubDAGs that are not the volume's own are refused, not silently replaced.
        cbq::SubDAGArray other = subDAGs;
        other[0].node_height += 1;
        try {
            (void)cbq::intersectVolume(vol, other, rays[0], rays[1], rays[2], rays[3], rays[4], rays[5], true);
            std::fprintf(stderr, "mismatched SubDAGs were accepted\n");
            return 5;
        } catch (const cbq::Error& e) {
            if (e.status != CBQ_ERR_INVALID_ARGUMENT) return 6;
        }
        std::vector<float> o, d;
        for (size_t i = half; i < n; i++) {
            o.insert(o.end(), &rays[6 * i], &rays[6 * i] + 3);
            d.insert(d.end(), &rays[6 * i + 3], &rays[6 * i + 3] + 3);
        }
        cbq::intersectVolumes(vol, o.data(), d.data(), n - half, true, cbq::MAX_FOOTPRINT_DISABLED, out.data() + half);
        cbq_free(nodes);
        FILE* g = std::fopen(argv[3], "wb");
        if (!g) return 4;
        std::fwrite(out.data(), sizeof(cbq::RayVolumeIntersection), n, g);
        std::fclose(g);
    } catch (const cbq::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
