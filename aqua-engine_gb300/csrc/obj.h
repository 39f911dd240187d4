// obj.h — Wavefront OBJ/MTL import into the scene format the loaders read
// (the role the reference's tobj-based conversion played, Cargo.toml:23:
// scenes/CornellBox-Original.obj -> scenes/CornellBox-Original_*.mesh +
// scenes/cbox.json), and the film writers (PFM, PPM).
#pragma once

#include <string>

namespace aq {

struct ObjConvertResult {
    int meshes = 0, triangles = 0, materials = 0;
};

// Reads `obj_path` and the MTL libraries it names; writes one BSON .mesh per
// OBJ group (`<stem>_<group>_<k>.mesh`: name, vertices, normals, texcoords,
// indices) and `out_dir/scene_name` (named_bsdfs, camera, lights, shapes).
// Throws SceneError (IO, PARSE).
ObjConvertResult convert_obj(const std::string& obj_path, const std::string& out_dir,
                             const std::string& scene_name, int width, int height);

// W x H x 3 floats, row 0 at the top. ".pfm": little-endian float PFM
// (rows bottom to top, as the format stores them); ".ppm": 8-bit P6 of the
// sRGB-encoded, clamped film. Throws SceneError.
void write_image(const std::string& path, const float* rgb, int w, int h);

}  // namespace aq
