/*
 * rtcore_scene.h -- seeded synthetic scenes and ray sets (host memory).
 *
 * The reference sample hard-codes one quad scene (vulkan-raytraced-triangle/
 * main.cpp:676-695, 835-858).  The workloads this core is measured on are
 * synthetic and seeded; these generators produce them identically on every
 * host: they use PCG32 (O'Neill 2014) streams and only the correctly rounded
 * IEEE operations + - * / sqrt, so x86-64 and aarch64 give the same bits.
 */
#ifndef RTCORE_SCENE_H
#define RTCORE_SCENE_H

#include "rtcore.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Surface material of the path-tracing scenes (Lambertian + emission). */
typedef struct rt_material {
    float albedo[3];
    float emission[3];
} rt_material;

/* Triangle soup: n_tris triangles, centroids uniform in [0,1]^3, two edge
 * vectors with directions uniform on the sphere and lengths ~U(0.001, 0.02);
 * v0 = c - (e1 + e2) / 3, v1 = v0 + e1, v2 = v0 + e2.  Unshared vertices:
 * vertices holds 9 * n_tris floats, indices 3 * n_tris (0, 1, 2, ...). */
rt_status rt_scene_soup(uint64_t seed, uint32_t n_tris, float *vertices, uint32_t *indices);

/* Closed box [-1,1]^3 (12 triangles: white floor/ceiling/back/front 0.73,
 * red left wall (0.65,0.05,0.05), green right wall (0.12,0.45,0.15)), a
 * 0.5 x 0.5 ceiling light of radiance 15 facing -y (2 triangles) and
 * n_spheres class-I geodesic icospheres of frequency freq (20 * freq^2
 * triangles each), radii ~U(0.05,0.25), centres ~U[-0.75,0.75]^3, albedo
 * ~U(0.1,0.9)^3.  Counts first, then the arrays. */
rt_status rt_scene_box_counts(uint32_t n_spheres, uint32_t freq, uint32_t *n_vertices, uint32_t *n_tris,
                              uint32_t *n_materials);
rt_status rt_scene_box(uint64_t seed, uint32_t n_spheres, uint32_t freq, float *vertices, uint32_t *indices,
                       uint32_t *tri_material, rt_material *materials);

/* n rays with origins uniform in the box [lo, hi] and directions uniform on
 * the unit sphere, tmin 0, the given tmax. */
rt_status rt_scene_incoherent_rays(uint64_t seed, uint32_t n, const float lo[3], const float hi[3], float tmax,
                                   rt_ray *rays);

/* Wavefront OBJ mesh (host files): counts first, then the arrays.
 * `v x y z` vertices (further numbers on the line ignored); `f` faces of three
 * or more references a, a/t, a//n or a/t/n (1-based, negative = relative to
 * the vertices read so far) split into the fan (a0, ai, ai+1); `usemtl name`
 * selects the material of the following faces, numbered 0, 1, ... in the order
 * faces first use them (faces before any usemtl use an unnamed material);
 * every other statement is skipped.  vertices: 3 floats per vertex; indices:
 * 3 per triangle; tri_material (nullable): one per triangle.  A missing file,
 * a malformed number or a reference outside the vertices gives
 * RT_ERR_INVALID_ARG.  No counterpart in the reference, which hard-codes its
 * arrays (vulkan-raytraced-triangle/main.cpp:676-682). */
rt_status rt_obj_counts(const char *path, uint32_t *n_vertices, uint32_t *n_tris, uint32_t *n_materials);
rt_status rt_obj_load(const char *path, float *vertices, uint32_t *indices, uint32_t *tri_material);

#ifdef __cplusplus
}
#endif
#endif
