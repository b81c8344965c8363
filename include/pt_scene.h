/*
 * pt_scene.h — C ABI of the host-side scene front end in libptgpu.so.
 *
 * Above the device boundary of pt_gpu.h sits the reference's CPU scene path:
 * the .scn parser (src/scene/scenebuild.cpp:132-365), per-object model import
 * (src/scene/scene.cpp:533-568, glTF 2.0 here), scene packing
 * (src/scene/scenebuffer.cpp:65-168), light-sampler tables
 * (src/scene/lightsample.cpp:89-221) and the camera matrix chain
 * (src/scene/camera.h:16, camera.cpp:21-26, pathtrace.cpp:381-396).
 * These calls replace SceneBuilder::read_scene_description + Scene +
 * SceneBuffer for a caller that wants to drive pt_gpu.h from scene files.
 */
#ifndef PT_SCENE_H_INCLUDED
#define PT_SCENE_H_INCLUDED

#include "pt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The reference's in-memory Scene (src/scene/scene.h:13-67) in flat arrays.
 * Mesh i is object variant i (one variant per mesh, scene.cpp:398-410); its
 * instances are instance_matrices[mesh_instance_offset[i] .. [i+1]). */
typedef struct pt_raw_scene {
    const float* vertices; /* PT_VERTEX_FLOATS per vertex, all meshes */
    uint32_t vertex_count;
    const uint32_t* indices; /* mesh-local, 3 per triangle */
    uint32_t index_count;
    const pt_mesh_range* meshes;
    const uint32_t* mesh_material;        /* material of each mesh/variant  */
    const uint32_t* mesh_instance_offset; /* mesh_count + 1 entries          */
    uint32_t mesh_count;
    const float* instance_matrices; /* 16 floats each, column-major (glm Mat4) */
    uint32_t instance_count;
    const pt_material* materials;
    uint32_t material_count;
    const float* point_lights; /* 6 floats each: position xyz, colour rgb */
    uint32_t point_light_count;
    const float* directional_lights; /* 6 floats each: direction, colour */
    uint32_t directional_light_count;
    float environment_colour[3];
    /* Textures (see pt_texture in pt_gpu.h); materials name them by index. */
    const uint8_t* texels;
    uint64_t texel_bytes;
    const pt_texture* textures;
    uint32_t texture_count;
    /* Optional (NULL = none), material_count entries: an index of refraction
     * > 0 makes the material a smooth refractive dielectric (see
     * pt_scene_view.material_ior); 0 keeps the reference's BSDF. */
    const float* material_ior;
} pt_raw_scene;

/* Camera description as parsed from a .scn camera section
 * (scenebuild.cpp:132-191); fov in degrees. */
typedef struct pt_camera_desc {
    float position[3];
    float lookdir[3];
    float up[3];
    float fov_degrees;
    float near_plane;
    float far_plane;
    float focus_dist;
    float lens_radius;
    float exposure;
} pt_camera_desc;

typedef struct pt_host_scene pt_host_scene;

/* Thread-local message of the last failing pt_scene_* call. */
const char* pt_scene_last_error(void);

/* Parse a .scn file and import its objects (SceneBuilder::read_scene_description,
 * scenebuild.cpp:279-365).  Returns NULL on error. */
pt_host_scene* pt_scene_load(const char* scn_path);

/* Build a scene from raw arrays (copied). */
pt_host_scene* pt_scene_from_raw(const pt_raw_scene* raw, const pt_camera_desc* camera);

void pt_scene_free(pt_host_scene* scene);

/* Borrow the raw arrays of a scene (valid until pt_scene_free). */
int pt_scene_raw(const pt_host_scene* scene, pt_raw_scene* out);

/* Camera of the scene (defaults of scenebuild.cpp:138-144 if none given). */
int pt_scene_camera(const pt_host_scene* scene, pt_camera_desc* out);

/* Pack the scene for the device (SceneBuffer::build + TableLightSampler) and
 * borrow the packed view (valid until pt_scene_free). */
int pt_scene_pack(pt_host_scene* scene, pt_scene_view* out);

/* Camera matrices and UBO fields for an image of width x height
 * (main.cpp:98 aspect = w/h; PathTracer::set_camera, pathtrace.cpp:381-396).
 * Fills inv_view, inv_proj, near/far, focus_dist, lens_radius, exposure,
 * width and height of `params`; leaves the other fields untouched. */
int pt_camera_params(const pt_camera_desc* camera, uint32_t width, uint32_t height,
                     pt_render_params* params);

/* sRGB decode as the reference applies it to colours read from scene files
 * (src/colour.cpp:12-14). */
float pt_from_srgb(float x);

/* One-line scene summary in the reference's format (scene.cpp:490-518). */
int pt_scene_details(const pt_host_scene* scene, char* buf, size_t buf_len);

/* Image writers of the reference's output stage (src/io/imagewrite.cpp:19-67):
 * Radiance RGBE .hdr of the RGB channels, and 8-bit RGBA PNG with the
 * truncating quantiser clamp(x*255) -> u8. */
int pt_write_hdr(const char* path, const float* rgba, uint32_t width, uint32_t height);
int pt_write_png(const char* path, const float* rgba, uint32_t width, uint32_t height);

/* Read a Radiance .hdr into RGBA floats (alpha = 1), decoded as m * 2^(e-136)
 * like the stb_image reader util/meansq uses; *rgba is malloc'ed, release it
 * with pt_host_free. */
int pt_read_hdr(const char* path, float** rgba, uint32_t* width, uint32_t* height);

/* Decodes a PNG image as the reference's texture loader keeps it (stb_image
 * with the file's channel count, 3 widened to 4; texturedata.cpp:30-48):
 * *texels (release with pt_host_free) holds width * height * channels bytes,
 * rows from the top.  *file_channels is the file's own channel count. */
int pt_png_decode(const uint8_t* data, size_t size, uint8_t** texels, uint32_t* width, uint32_t* height,
                  uint32_t* channels, uint32_t* file_channels);

/* Decodes a baseline (sequential Huffman, 8-bit) JPEG image as the
 * reference's texture loader keeps it (stb_image, texturedata.cpp:30-48): 1
 * channel for greyscale files, 4 (RGB + alpha 255) for colour files; rows from
 * the top; release *texels with pt_host_free.  Texels may differ from
 * stb_image's by a few units (its integer IDCT and fixed-point colour
 * conversion round differently).  Progressive, lossless and arithmetic-coded
 * files are refused with PT_ERR_IO. */
int pt_jpeg_decode(const uint8_t* data, size_t size, uint8_t** texels, uint32_t* width, uint32_t* height,
                   uint32_t* channels, uint32_t* file_channels);

/* Release memory returned by pt_read_hdr, pt_png_decode and pt_jpeg_decode. */
void pt_host_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* PT_SCENE_H_INCLUDED */
