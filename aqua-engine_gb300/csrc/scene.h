// scene.h — host-side scene: the triangles, materials, lights, textures and
// camera the renderer consumes, and the loaders that fill it.
//
// Loaders follow the reference's data contract:
//   scene JSON     scenes/cbox.json:1-628, scenes/room.json:1-3900
//                  (named_bsdfs / camera / lights / shapes, serde externally
//                  tagged enums: Principled, Perspective, Point, Mesh, Named,
//                  Float / Float3 / Srgb / Image)
//   integrator     scenes/integrator.json:1-9
//   BSON .mesh     scenes/*.mesh: {name, vertices[[f64x3]], normals[[f64x3]],
//                  texcoords[[f64x2]], indices[[i64x3]]}
// Procedural scenes 1-5 are the seeded synthetic workloads the benchmarks use.
#pragma once

#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/aqua.h"

namespace aq {

struct Texture {
    int w = 0, h = 0;
    std::vector<uint8_t> rgba;  // sRGB-encoded RGBA8, row-major
};

struct HostScene {
    std::vector<float> verts;      // 9 floats per triangle, scene order
    std::vector<float> uvs;        // 6 floats per triangle (zeros when absent)
    std::vector<float> nrm;        // 9 floats per triangle: vertex normals (scene order), or
                                   // empty when no mesh of the scene carries normals
    std::vector<int32_t> tri_mat;  // material per triangle
    std::vector<int32_t> tri_light;  // light the triangle belongs to, or -1
    std::vector<aqua_material> mats;
    std::vector<std::string> mat_names;
    std::vector<aqua_light> lights;
    std::vector<Texture> textures;
    aqua_camera cam{};
    float env[3] = {0, 0, 0};
    int num_meshes = 0;
    size_t num_tris() const { return tri_mat.size(); }
};

struct SceneError : std::runtime_error {
    aqua_status status;
    SceneError(aqua_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

struct MeshData {
    std::string name;
    std::vector<double> positions;  // 3 per vertex
    std::vector<double> normals;    // 3 per vertex or empty
    std::vector<double> texcoords;  // 2 per vertex or empty
    std::vector<int64_t> indices;   // 3 per triangle
};

// BSON .mesh reader (bsonspec.org v1.1 subset: document, array, string,
// double, int32, int64). Throws SceneError(IO / PARSE).
MeshData read_mesh_bson(const std::string& path);
MeshData parse_mesh_bson(const uint8_t* data, size_t n);

// Throws SceneError.
HostScene load_scene_json(const std::string& path, bool allow_missing);
void load_integrator_json(const std::string& path, aqua_integrator_cfg* cfg);
HostScene make_procedural(int config_id, uint64_t seed, int width, int height);

// Camera from a Perspective block: TRS with Euler rotation in degrees,
// applied X, then Y, then Z; the camera looks down its local -z axis.
aqua_camera make_camera(int w, int h, float fov_deg, float lens_radius, float focal,
                        const double translate[3], const double rotate_deg[3]);
void camera_look_at(aqua_camera& c, const float eye[3], const float target[3], const float up[3]);

// Recomputes the power-weighted selection pmf of every light.
void finalize_lights(HostScene& s);

// Deterministic elementary functions built from + - * / only, so that
// procedural scenes are bit-identical on every host.
double det_sin(double x);
double det_cos(double x);
double det_exp(double x);
double det_log(double x);

}  // namespace aq
