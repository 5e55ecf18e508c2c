// rt_sample -- headless drop-in for the reference's ray-tracing sample
// (vulkan-raytraced-triangle/main.cpp == vulkan-raytracing-basic/main.cpp).
//
// main() of the sample (main.cpp:1425-1454) creates a window and a Vulkan
// device, builds a BLAS and a TLAS, an output image, a camera uniform, the
// ray-tracing pipeline and its shader binding table, then renders frames into
// the swapchain.  This program runs the same sequence through the C ABI of
// librtcore, without a window: one frame (or --frames N timed frames) into an
// RGBA32F device buffer, written out as PPM (and PFM).
//
//   rt_sample [--scene ref8|tri] [--obj F.obj] [--camera X Y Z FOV]
//             [--width W] [--height H] [--out F.ppm] [--pfm F.pfm]
//             [--raw F.bin] [--frames N]
//
// --scene ref8: the sample's own scene and camera (1200x800, camera (0,0,10),
//               two geometries x two instances, SBT colours, sample chit);
// --scene tri : one triangle (-1,-1,0),(1,-1,0),(0,1,0), camera (0,0,2.5),
//               800x600, barycentric closest hit.
// --obj F     : the mesh of a Wavefront OBJ file (rt_obj_load) as one
//               geometry under one identity instance, barycentric closest
//               hit, 800x600; the camera looks down -z at the mesh from in
//               front of its bounds unless --camera gives it.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rtcore.h"
#include "rtcore_scene.h"

namespace {

#define CHECK_RT(expr)                                                                          \
    do {                                                                                        \
        rt_status s_ = (expr);                                                                  \
        if (s_ != RT_OK) {                                                                      \
            std::fprintf(stderr, "%s failed: %d (%s)\n", #expr, s_, rt_last_error_string(ctx)); \
            return 1;                                                                           \
        }                                                                                       \
    } while (0)
#define CHECK_CUDA(expr)                                                                  \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            std::fprintf(stderr, "%s failed: %s\n", #expr, cudaGetErrorString(e_));       \
            return 1;                                                                     \
        }                                                                                 \
    } while (0)

template <class T>
T *upload(const T *host, size_t n) {
    void *d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * (n ? n : 1)) != cudaSuccess) return nullptr;
    if (n) cudaMemcpy(d, host, sizeof(T) * n, cudaMemcpyHostToDevice);
    return static_cast<T *>(d);
}

}  // namespace

int main(int argc, char **argv) {
    std::string scene = "ref8", out_ppm = "rt_sample.ppm", out_pfm, out_raw, obj;
    uint32_t width = 0, height = 0;
    bool cam_given = false;
    float cam_arg[4] = {0.0f, 0.0f, 0.0f, 60.0f};
    int frames = 1;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> const char * { return i + 1 < argc ? argv[++i] : ""; };
        if (a == "--scene") scene = next();
        else if (a == "--width") width = (uint32_t)std::atoi(next());
        else if (a == "--height") height = (uint32_t)std::atoi(next());
        else if (a == "--out") out_ppm = next();
        else if (a == "--pfm") out_pfm = next();
        else if (a == "--raw") out_raw = next();
        else if (a == "--frames") frames = std::atoi(next());
        else if (a == "--obj") { obj = next(); scene = "obj"; }
        else if (a == "--camera") {
            for (int k = 0; k < 4; ++k) cam_arg[k] = (float)std::atof(next());
            cam_given = true;
        }
        else {
            std::fprintf(stderr, "unknown argument %s\n", a.c_str());
            return 2;
        }
    }
    const bool ref8 = scene == "ref8";
    if (!ref8 && scene != "tri" && scene != "obj") {
        std::fprintf(stderr, "--scene must be ref8 or tri\n");
        return 2;
    }
    if (!width) width = ref8 ? 1200u : 800u;   // main.cpp:13-14
    if (!height) height = ref8 ? 800u : 600u;

    rt_context *ctx = nullptr;
    {
        rt_status s = rt_context_create(0, &ctx);
        if (s != RT_OK) {
            std::fprintf(stderr, "rt_context_create failed: %d\n", s);
            return 1;
        }
    }
    cudaStream_t stream;
    CHECK_CUDA(cudaStreamCreate(&stream));

    // ---- createBLAS (main.cpp:674-831)
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    std::vector<rt_transform3x4> geo_xf;
    if (ref8) {
        vertices = {-1, -1, 0, 1, -1, 0, 1, 1, 0, -1, 1, 0};          // main.cpp:676-681
        indices = {0, 1, 3, 1, 2, 3};                                  // main.cpp:682
        geo_xf = {{{{1, 0, 0, -2}, {0, 1, 0, 0}, {0, 0, 1, 0}}},       // main.cpp:684-695
                  {{{1, 0, 0, 2}, {0, 1, 0, 0}, {0, 0, 1, 0}}}};
    } else if (scene == "obj") {
        uint32_t nv = 0, nt = 0, nm = 0;
        rt_status s = rt_obj_counts(obj.c_str(), &nv, &nt, &nm);
        if (s == RT_OK) {
            vertices.resize((size_t)nv * 3u);
            indices.resize((size_t)nt * 3u);
            s = rt_obj_load(obj.c_str(), vertices.data(), indices.data(), nullptr);
        }
        if (s != RT_OK || nt == 0) {
            std::fprintf(stderr, "cannot load %s as an OBJ mesh with triangles (%d)\n", obj.c_str(), s);
            return 1;
        }
        if (!cam_given) {
            // in front of the bounds (+z), looking -z, 60 degrees
            float lo[3] = {vertices[0], vertices[1], vertices[2]}, hi[3] = {lo[0], lo[1], lo[2]};
            for (size_t k = 0; k < vertices.size(); ++k) {
                lo[k % 3] = vertices[k] < lo[k % 3] ? vertices[k] : lo[k % 3];
                hi[k % 3] = vertices[k] > hi[k % 3] ? vertices[k] : hi[k % 3];
            }
            const float ext = (hi[0] - lo[0]) > (hi[1] - lo[1]) ? (hi[0] - lo[0]) : (hi[1] - lo[1]);
            cam_arg[0] = 0.5f * (lo[0] + hi[0]);
            cam_arg[1] = 0.5f * (lo[1] + hi[1]);
            cam_arg[2] = hi[2] + 1.2f * ext;
            cam_arg[3] = 60.0f;
        }
    } else {
        vertices = {-1, -1, 0, 1, -1, 0, 0, 1, 0};
        indices = {0, 1, 2};
    }
    float *d_vert = upload(vertices.data(), vertices.size());
    uint32_t *d_idx = upload(indices.data(), indices.size());
    rt_transform3x4 *d_xf = geo_xf.empty() ? nullptr : upload(geo_xf.data(), geo_xf.size());
    if (!d_vert || !d_idx || (!geo_xf.empty() && !d_xf)) {
        std::fprintf(stderr, "device allocation failed\n");
        return 1;
    }
    const uint32_t n_geoms = ref8 ? 2u : 1u;
    rt_geometry_triangles geoms[2];
    for (uint32_t g = 0; g < n_geoms; ++g) {
        geoms[g].vertices = d_vert;
        geoms[g].vertex_stride = 12;                           // sizeof(vertices[0])
        geoms[g].max_vertex = (uint32_t)(vertices.size() / 3 - 1);
        geoms[g].index_type = RT_INDEX_UINT32;
        geoms[g].indices = d_idx;
        geoms[g].tri_count = (uint32_t)(indices.size() / 3);
        geoms[g].flags = RT_GEOMETRY_OPAQUE;
        geoms[g].transform = d_xf ? d_xf + g : nullptr;       // transformOffset 0 / 48 B
    }
    uint32_t counts[2] = {geoms[0].tri_count, geoms[1 % n_geoms].tri_count};
    rt_build_sizes bs;
    CHECK_RT(rt_get_blas_build_sizes(ctx, counts, n_geoms, RT_BUILD_PREFER_FAST_TRACE, &bs));
    void *blas = nullptr, *scratch = nullptr;
    CHECK_CUDA(cudaMalloc(&blas, bs.accel_bytes));
    CHECK_CUDA(cudaMalloc(&scratch, bs.scratch_bytes));
    CHECK_RT(rt_build_blas(ctx, stream, geoms, n_geoms, RT_BUILD_PREFER_FAST_TRACE, blas, bs.accel_bytes, scratch,
                           bs.scratch_bytes));
    CHECK_RT(rt_sync(ctx, stream));
    cudaFree(scratch);

    // ---- createTLAS (main.cpp:833-949)
    std::vector<rt_instance> inst;
    auto make_inst = [&](float ty, uint32_t sbt_offset) {
        rt_instance I;
        std::memset(&I, 0, sizeof(I));
        const float m[3][4] = {{1, 0, 0, 0}, {0, 1, 0, ty}, {0, 0, 1, 0}};
        std::memcpy(I.transform.m, m, sizeof(m));
        I.custom_index_and_mask = (ref8 ? 100u : 0u) | (0xffu << 24);           // main.cpp:850-851
        I.sbt_offset_and_flags = sbt_offset | (1u << 24);                         // FACING_CULL_DISABLE
        I.accel_ref = rt_accel_address(blas);
        return I;
    };
    if (ref8) {
        inst.push_back(make_inst(2.0f, 0));   // main.cpp:835-840
        inst.push_back(make_inst(-2.0f, 2));  // main.cpp:841-846, 857
    } else {
        inst.push_back(make_inst(0.0f, 0));
    }
    rt_instance *d_inst = upload(inst.data(), inst.size());
    CHECK_RT(rt_get_tlas_build_sizes(ctx, (uint32_t)inst.size(), RT_BUILD_PREFER_FAST_TRACE, &bs));
    void *tlas = nullptr;
    CHECK_CUDA(cudaMalloc(&tlas, bs.accel_bytes));
    CHECK_CUDA(cudaMalloc(&scratch, bs.scratch_bytes));
    CHECK_RT(rt_build_tlas(ctx, stream, d_inst, (uint32_t)inst.size(), RT_BUILD_PREFER_FAST_TRACE, tlas,
                           bs.accel_bytes, scratch, bs.scratch_bytes));
    CHECK_RT(rt_sync(ctx, stream));
    cudaFree(scratch);

    // ---- createOutImage (main.cpp:951-999): RGBA32F storage buffer
    float *d_img = nullptr;
    CHECK_CUDA(cudaMalloc(&d_img, (size_t)width * height * 16u));

    // ---- createUniformBuffer (main.cpp:1001-1017)
    rt_camera cam = ref8 ? rt_camera{{0.0f, 0.0f, 10.0f}, 60.0f} : rt_camera{{0.0f, 0.0f, 2.5f}, 60.0f};
    if (scene == "obj" || cam_given) cam = rt_camera{{cam_arg[0], cam_arg[1], cam_arg[2]}, cam_arg[3]};

    // ---- createRayTracingPipeline + createShaderBindingTable (main.cpp:1093-1320)
    rt_pipeline pipe;
    std::memset(&pipe, 0, sizeof(pipe));
    pipe.chit = ref8 ? RT_CHIT_SAMPLE : RT_CHIT_BARYCENTRIC;
    pipe.ray_flags = RT_RAY_FLAG_OPAQUE;
    pipe.cull_mask = 0xff;
    pipe.sbt_record_offset = 0;
    pipe.sbt_record_stride = 1;
    pipe.miss_index = 0;
    pipe.tmin = 0.0f;
    pipe.tmax = 100.0f;
    pipe.miss_color[0] = 0.0f; pipe.miss_color[1] = 0.0f; pipe.miss_color[2] = 0.2f;
    pipe.max_recursion = 1;
    const float colors[12] = {0.6f, 0.1f, 0.2f, 0.1f, 0.8f, 0.4f,   // main.cpp:1310-1317
                              0.9f, 0.7f, 0.1f, 0.3f, 0.6f, 0.9f};
    float *d_sbt = upload(colors, 12);
    rt_sbt sbt{d_sbt, 4u, 3u};

    // ---- render (main.cpp:1322-1423): vkCmdTraceRaysKHR(..., W, H, 1)
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    CHECK_RT(rt_trace_rays(ctx, stream, &pipe, &sbt, rt_accel_address(tlas), &cam, d_img, width, height, 1));
    CHECK_RT(rt_sync(ctx, stream));
    if (frames > 1) {
        cudaEventRecord(e0, stream);
        for (int f = 0; f < frames; ++f)
            CHECK_RT(rt_trace_rays(ctx, stream, &pipe, &sbt, rt_accel_address(tlas), &cam, d_img, width, height, 1));
        cudaEventRecord(e1, stream);
        CHECK_RT(rt_sync(ctx, stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        std::printf("{\"frames\": %d, \"ms_per_frame\": %.4f, \"mrays_per_s\": %.2f}\n", frames, ms / frames,
                    (double)width * height * frames / (ms * 1e3));
    }
    std::vector<float> img((size_t)width * height * 4u);
    CHECK_CUDA(cudaMemcpy(img.data(), d_img, img.size() * 4u, cudaMemcpyDeviceToHost));
    CHECK_RT(rt_write_ppm(img.data(), width, height, out_ppm.c_str()));
    if (!out_pfm.empty()) CHECK_RT(rt_write_pfm(img.data(), width, height, out_pfm.c_str()));
    if (!out_raw.empty()) {
        FILE *f = std::fopen(out_raw.c_str(), "wb");
        if (!f || std::fwrite(img.data(), 4, img.size(), f) != img.size()) {
            std::fprintf(stderr, "cannot write %s\n", out_raw.c_str());
            return 1;
        }
        std::fclose(f);
    }
    std::printf("wrote %s (%ux%u)\n", out_ppm.c_str(), width, height);

    cudaFree(d_img);
    cudaFree(d_sbt);
    cudaFree(tlas);
    cudaFree(blas);
    cudaFree(d_inst);
    cudaFree(d_vert);
    cudaFree(d_idx);
    if (d_xf) cudaFree(d_xf);
    cudaStreamDestroy(stream);
    rt_context_destroy(ctx);
    return 0;
}
