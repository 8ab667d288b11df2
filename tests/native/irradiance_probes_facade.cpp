// A C++ host program of the kind VulkanExp's editor is, driving the probe
// update through include/irradiance_probes.hpp (the IrradianceProbes class
// over the C ABI).  Used by tests/test_facade.py: the test writes a scene, a
// grid, a light and a sequence of rotations to a folder, runs this program on
// it, and compares what it writes with the same sequence driven through the
// Python mirror.
//
//   irradiance_probes_facade <folder>
//
// Reads grid.bin (ddgi_grid_desc), light.bin (ddgi_light), params.bin
// (uint32 updates, uint32 ProbesPerUpdate, float TargetHysteresis), orient.bin
// ((updates + 1) x 9 floats: initProbes first), and the scene arrays
// vertices.bin, indices.bin, meshes.bin, instances.bin, offsets.bin,
// materials.bin.  Writes out.bin: per update the blended and the host-side
// hysteresis (2 floats), then the colour atlas, the depth atlas (floats) and
// the probe states (uint32).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "irradiance_probes.hpp"

namespace {

std::vector<char> slurp(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot read " + path);
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

template <class T>
std::vector<T> array_of(const std::string& path) {
    std::vector<char> b = slurp(path);
    std::vector<T> v(b.size() / sizeof(T));
    if (!v.empty()) std::memcpy(v.data(), b.data(), v.size() * sizeof(T));
    return v;
}

template <class T>
T one_of(const std::string& path) {
    std::vector<T> v = array_of<T>(path);
    if (v.size() != 1) throw std::runtime_error("bad size of " + path);
    return v[0];
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s <folder>\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    try {
        const ddgi_grid_desc grid = one_of<ddgi_grid_desc>(dir + "/grid.bin");
        const ddgi_light light = one_of<ddgi_light>(dir + "/light.bin");
        const std::vector<uint32_t> params = array_of<uint32_t>(dir + "/params.bin");
        if (params.size() != 3) throw std::runtime_error("bad params.bin");
        const uint32_t updates = params[0];
        float target;
        std::memcpy(&target, &params[2], 4);
        const std::vector<float> orient = array_of<float>(dir + "/orient.bin");
        if (orient.size() != 9 * (size_t)(updates + 1)) throw std::runtime_error("bad orient.bin");
        const auto vertices = array_of<ddgi_vertex>(dir + "/vertices.bin");
        const auto indices = array_of<uint32_t>(dir + "/indices.bin");
        const auto meshes = array_of<ddgi_mesh>(dir + "/meshes.bin");
        const auto instances = array_of<ddgi_instance>(dir + "/instances.bin");
        const auto offsets = array_of<ddgi_offset_entry>(dir + "/offsets.bin");
        const auto materials = array_of<ddgi_material>(dir + "/materials.bin");
        ddgi_scene_desc scene{};
        scene.vertices = vertices.data();
        scene.vertex_count = (uint32_t)vertices.size();
        scene.indices = indices.data();
        scene.index_count = (uint32_t)indices.size();
        scene.meshes = meshes.data();
        scene.mesh_count = (uint32_t)meshes.size();
        scene.instances = instances.data();
        scene.instance_count = (uint32_t)instances.size();
        scene.offsets = offsets.data();
        scene.offset_count = (uint32_t)offsets.size();
        scene.materials = materials.data();
        scene.material_count = (uint32_t)materials.size();

        // the editor's sequence: configure, init, bind, classify, update
        ddgi::IrradianceProbes probes;
        probes.GridParameters = grid;
        probes.ProbesPerUpdate = params[1];
        probes.TargetHysteresis = target;
        probes.init(grid.extent_min, grid.extent_max);
        probes.writeDescriptorSet(scene, light);
        probes.initProbes(orient.data(), nullptr);
        std::vector<float> ramp;
        for (uint32_t k = 0; k < updates; ++k) {
            probes.update(orient.data() + 9 * (size_t)(k + 1), nullptr);
            ramp.push_back(probes.blendedHysteresis());
            ramp.push_back(probes.currentHysteresis());
        }
        uint32_t cw, ch, cc, dw, dh, dc;
        ddgi_ctx* ctx = probes.context();
        if (ddgi_atlas_dims(ctx, DDGI_ATLAS_COLOR, &cw, &ch, &cc) != DDGI_OK ||
            ddgi_atlas_dims(ctx, DDGI_ATLAS_DEPTH, &dw, &dh, &dc) != DDGI_OK)
            throw std::runtime_error("ddgi_atlas_dims");
        std::vector<float> color((size_t)cw * ch * cc), depth((size_t)dw * dh * dc);
        std::vector<uint32_t> states(probes.getProbeCount());
        if (ddgi_get_atlas(ctx, DDGI_ATLAS_COLOR, color.data(), color.size() * 4, nullptr) != DDGI_OK ||
            ddgi_get_atlas(ctx, DDGI_ATLAS_DEPTH, depth.data(), depth.size() * 4, nullptr) != DDGI_OK ||
            ddgi_get_probe_states(ctx, states.data(), states.size(), nullptr) != DDGI_OK)
            throw std::runtime_error(std::string("read back: ") + ddgi_last_error(ctx));
        std::ofstream out(dir + "/out.bin", std::ios::binary);
        out.write(reinterpret_cast<const char*>(ramp.data()), ramp.size() * 4);
        out.write(reinterpret_cast<const char*>(color.data()), color.size() * 4);
        out.write(reinterpret_cast<const char*>(depth.data()), depth.size() * 4);
        out.write(reinterpret_cast<const char*>(states.data()), states.size() * 4);
        if (!out) throw std::runtime_error("cannot write out.bin");
        probes.destroy();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    std::printf("ok\n");
    return 0;
}
