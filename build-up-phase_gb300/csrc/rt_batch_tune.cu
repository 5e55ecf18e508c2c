// rt_batch_tune.cu -- autotuner of the batched path tracer (rtcore_batch.h)
// and its JSON cache.
//
// No counterpart in the reference: its launch shape is fixed by the driver
// (vkCmdTraceRaysKHR over WIDTH x HEIGHT, vulkan-raytraced-triangle/main.cpp:
// 1349-1355, :13-14).  Here the shapes of the software traversal and shading
// kernels -- traversal block size and blocks per SM, shared-memory stack
// depth, the refill threshold of the persistent warps, the shading block size
// and the wave size (queue capacity) -- are measured on the batch itself:
// coordinate descent from the defaults, one parameter at a time, each
// candidate timed as a graph launch of one sample per pixel (results
// discarded), best of three launches after a warm-up, CUDA events on the
// launching stream.  The winner is stored in a JSON file keyed by device,
// scene count, triangle count, pixel count and depth, so a later run of a
// batch of the same shape reuses it without tuning.
#include <cuda_runtime.h>

#include <cerrno>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include <unistd.h>

#include "../../include/rtcore_batch.h"
#include "rt_internal.h"

namespace {

// ---------------------------------------------------------------------------
// A small JSON reader/writer: objects, arrays, strings, numbers, literals.
// ---------------------------------------------------------------------------

struct Json {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    double num = 0.0;
    bool b = false;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json *get(const char *k) const {
        if (kind != Obj) return nullptr;
        for (const auto &kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

class Reader {
public:
    Reader(const char *p, const char *e) : p_(p), e_(e) {}
    bool document(Json &out) {
        if (!value(out, 0)) return false;
        ws();
        return p_ == e_;
    }

private:
    const char *p_, *e_;
    void ws() {
        while (p_ < e_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char *s) {
        const size_t n = std::strlen(s);
        if ((size_t)(e_ - p_) < n || std::strncmp(p_, s, n) != 0) return false;
        p_ += n;
        return true;
    }
    bool string(std::string &out) {
        if (p_ >= e_ || *p_ != '"') return false;
        ++p_;
        out.clear();
        while (p_ < e_ && *p_ != '"') {
            char c = *p_++;
            if (c == '\\') {
                if (p_ >= e_) return false;
                const char x = *p_++;
                switch (x) {
                case '"': c = '"'; break;
                case '\\': c = '\\'; break;
                case '/': c = '/'; break;
                case 'n': c = '\n'; break;
                case 't': c = '\t'; break;
                case 'r': c = '\r'; break;
                case 'b': c = '\b'; break;
                case 'f': c = '\f'; break;
                default: return false;  // \u escapes never occur in keys this file writes
                }
            } else if ((unsigned char)c < 0x20u) {
                return false;
            }
            out.push_back(c);
        }
        if (p_ >= e_) return false;
        ++p_;
        return true;
    }
    bool number(double &out) {
        const char *s = p_;
        if (p_ < e_ && (*p_ == '-' || *p_ == '+')) ++p_;
        bool digits = false;
        while (p_ < e_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' || *p_ == '-' ||
                           *p_ == '+')) {
            digits = digits || (*p_ >= '0' && *p_ <= '9');
            ++p_;
        }
        if (!digits || p_ - s > 63) return false;
        char buf[64];
        std::memcpy(buf, s, (size_t)(p_ - s));
        buf[p_ - s] = 0;
        char *end = nullptr;
        out = std::strtod(buf, &end);
        return end == buf + (p_ - s);
    }
    bool value(Json &v, int depth) {
        if (depth > 32) return false;
        ws();
        if (p_ >= e_) return false;
        const char c = *p_;
        if (c == '{') {
            ++p_;
            v.kind = Json::Obj;
            ws();
            if (p_ < e_ && *p_ == '}') { ++p_; return true; }
            for (;;) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (p_ >= e_ || *p_ != ':') return false;
                ++p_;
                Json x;
                if (!value(x, depth + 1)) return false;
                v.obj.emplace_back(std::move(k), std::move(x));
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == '}') { ++p_; return true; }
                return false;
            }
        }
        if (c == '[') {
            ++p_;
            v.kind = Json::Arr;
            ws();
            if (p_ < e_ && *p_ == ']') { ++p_; return true; }
            for (;;) {
                Json x;
                if (!value(x, depth + 1)) return false;
                v.arr.push_back(std::move(x));
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == ']') { ++p_; return true; }
                return false;
            }
        }
        if (c == '"') { v.kind = Json::Str; return string(v.str); }
        if (lit("true")) { v.kind = Json::Bool; v.b = true; return true; }
        if (lit("false")) { v.kind = Json::Bool; v.b = false; return true; }
        if (lit("null")) { v.kind = Json::Null; return true; }
        v.kind = Json::Num;
        return number(v.num);
    }
};

void write_string(std::string &o, const std::string &s) {
    o.push_back('"');
    for (char c : s) {
        if (c == '"' || c == '\\') { o.push_back('\\'); o.push_back(c); }
        else if (c == '\n') o += "\\n";
        else if (c == '\t') o += "\\t";
        else if ((unsigned char)c < 0x20u) o.push_back(' ');
        else o.push_back(c);
    }
    o.push_back('"');
}

void write_json(std::string &o, const Json &v, int indent) {
    const std::string pad((size_t)indent * 2u, ' '), pad2((size_t)(indent + 1) * 2u, ' ');
    switch (v.kind) {
    case Json::Null: o += "null"; break;
    case Json::Bool: o += v.b ? "true" : "false"; break;
    case Json::Num: {
        char buf[64];
        if (v.num == std::floor(v.num) && std::fabs(v.num) < 1e15) std::snprintf(buf, sizeof(buf), "%.0f", v.num);
        else std::snprintf(buf, sizeof(buf), "%.6g", v.num);
        o += buf;
        break;
    }
    case Json::Str: write_string(o, v.str); break;
    case Json::Arr: {
        // arrays of scalars on one line, others one element per line
        bool flat = true;
        for (const auto &x : v.arr) flat = flat && x.kind != Json::Obj && x.kind != Json::Arr;
        o.push_back('[');
        for (size_t i = 0; i < v.arr.size(); ++i) {
            if (!flat) { o.push_back('\n'); o += pad2; }
            write_json(o, v.arr[i], indent + 1);
            if (i + 1 < v.arr.size()) o += flat ? ", " : ",";
        }
        if (!flat && !v.arr.empty()) { o.push_back('\n'); o += pad; }
        o.push_back(']');
        break;
    }
    case Json::Obj: {
        o.push_back('{');
        for (size_t i = 0; i < v.obj.size(); ++i) {
            o.push_back('\n');
            o += pad2;
            write_string(o, v.obj[i].first);
            o += ": ";
            write_json(o, v.obj[i].second, indent + 1);
            if (i + 1 < v.obj.size()) o.push_back(',');
        }
        if (!v.obj.empty()) { o.push_back('\n'); o += pad; }
        o.push_back('}');
        break;
    }
    }
}

Json num(double x) {
    Json j;
    j.kind = Json::Num;
    j.num = x;
    return j;
}

Json str(const std::string &s) {
    Json j;
    j.kind = Json::Str;
    j.str = s;
    return j;
}

constexpr const char *kFormat = "rtcore-batch-tuning/1";

const char *const kFields[] = {"trace_threads", "trace_blocks_per_sm", "stack_ring", "refill",
                               "shade_threads", "wave_paths", "bvh_width"};

uint32_t *field(rt_batch_tuning &t, int i) {
    switch (i) {
    case 0: return &t.trace_threads;
    case 1: return &t.trace_blocks_per_sm;
    case 2: return &t.stack_ring;
    case 3: return &t.refill;
    case 4: return &t.shade_threads;
    case 5: return &t.wave_paths;
    default: return &t.bvh_width;
    }
}

Json tuning_json(const rt_batch_tuning &t, float ms) {
    Json o;
    o.kind = Json::Obj;
    rt_batch_tuning c = t;
    for (int i = 0; i < 7; ++i) o.obj.emplace_back(kFields[i], num(*field(c, i)));
    o.obj.emplace_back("ms", num(std::round((double)ms * 1000.0) / 1000.0));
    return o;
}

// 0: parsed; 1: no file; 2: unreadable or not a tuning cache
int read_cache(const char *path, Json &doc) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return 1;
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) {
        text.append(buf, n);
        if (text.size() > (64u << 20)) break;
    }
    std::fclose(f);
    Reader r(text.data(), text.data() + text.size());
    if (!r.document(doc) || doc.kind != Json::Obj) return 2;
    const Json *fmt = doc.get("format");
    const Json *ent = doc.get("entries");
    if (!fmt || fmt->kind != Json::Str || fmt->str != kFormat || !ent || ent->kind != Json::Obj) return 2;
    return 0;
}

uint32_t log2_bucket(uint64_t x) {
    uint32_t b = 0;
    while (x > 1u) {
        x >>= 1u;
        ++b;
    }
    return b;
}

}  // namespace

extern "C" rt_status rt_batch_tuning_cache_lookup(const char *path, const char *key, rt_batch_tuning *t, float *ms) {
    if (!path || !key || !t) return RT_ERR_INVALID_ARG;
    Json doc;
    const int rc = read_cache(path, doc);
    if (rc == 1) return RT_ERR_NOT_FOUND;
    if (rc == 2) return RT_ERR_INVALID_ARG;
    const Json *e = doc.get("entries")->get(key);
    if (!e || e->kind != Json::Obj) return RT_ERR_NOT_FOUND;
    rt_batch_tuning out;
    rt_batch_default_tuning(&out);
    for (int i = 0; i < 7; ++i) {
        const Json *v = e->get(kFields[i]);
        if (!v || v->kind != Json::Num || v->num < 0.0 || v->num > 4294967295.0 || v->num != std::floor(v->num))
            return RT_ERR_INVALID_ARG;
        *field(out, i) = (uint32_t)v->num;
    }
    *t = out;
    if (ms) {
        const Json *m = e->get("ms");
        *ms = (m && m->kind == Json::Num) ? (float)m->num : 0.0f;
    }
    return RT_OK;
}

namespace {

rt_status cache_store(const char *path, const char *key, const rt_batch_tuning *t, float ms, const Json *trials) {
    if (!path || !key || !t) return RT_ERR_INVALID_ARG;
    Json doc;
    const int rc = read_cache(path, doc);
    if (rc == 2) return RT_ERR_INVALID_ARG;  // never overwrite a file that is not a tuning cache
    if (rc == 1) {
        doc = Json();
        doc.kind = Json::Obj;
        doc.obj.emplace_back("format", str(kFormat));
        Json ent;
        ent.kind = Json::Obj;
        doc.obj.emplace_back("entries", ent);
    }
    Json *ent = nullptr;
    for (auto &kv : doc.obj)
        if (kv.first == "entries") ent = &kv.second;
    // a new entry, or the tuning fields and time of an existing one updated
    // in place (its other fields, such as earlier trials, kept)
    const Json e = tuning_json(*t, ms);
    Json *old = nullptr;
    for (auto &kv : ent->obj)
        if (kv.first == key && kv.second.kind == Json::Obj) old = &kv.second;
    if (!old) {
        ent->obj.emplace_back(key, Json());
        old = &ent->obj.back().second;
        old->kind = Json::Obj;
    }
    auto put = [&](const std::string &k, const Json &v) {
        for (auto &kv : old->obj)
            if (kv.first == k) {
                kv.second = v;
                return;
            }
        old->obj.emplace_back(k, v);
    };
    for (const auto &kv : e.obj) put(kv.first, kv.second);
    if (trials) put("trials", *trials);
    std::string text;
    write_json(text, doc, 0);
    text.push_back('\n');
    const std::string tmp = std::string(path) + ".tmp." + std::to_string((long)getpid());
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return RT_ERR_INVALID_ARG;
    const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
    if (std::fclose(f) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return RT_ERR_INVALID_ARG;
    }
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_batch_tuning_cache_store(const char *path, const char *key, const rt_batch_tuning *t,
                                                 float ms) {
    return cache_store(path, key, t, ms, nullptr);
}

extern "C" rt_status rt_batch_tuning_key(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n_scenes,
                                         const rt_batch_params *p, char *key, uint32_t key_bytes) {
    if (!ctx || !p || !key || key_bytes == 0 || (n_scenes && !scenes))
        return rtc::set_error(ctx, RT_ERR_INVALID_ARG, "rt_batch_tuning_key: null argument");
    RT_CUDA_CTX(ctx, cudaSetDevice(ctx->device));
    uint64_t tris = 0, pixels = 0;
    for (uint32_t s = 0; s < n_scenes; ++s) {
        const uint64_t npix = (uint64_t)scenes[s].width * scenes[s].height;
        if (!npix || !scenes[s].scene.accel) continue;
        pixels += npix;
        uint32_t prims = 0;
        const void *src = reinterpret_cast<const uint8_t *>(scenes[s].scene.accel) + offsetof(rt_accel_header, prim_count);
        RT_CUDA_CTX(ctx, cudaMemcpy(&prims, src, sizeof(prims), cudaMemcpyDeviceToHost));
        tris += prims;
    }
    // (the key does not depend on the width the structures were built with:
    // the width is one of the tuned choices stored under it)
    const int n = std::snprintf(key, key_bytes, "sm%d%d-%d/n2^%u/tris2^%u/px2^%u/d%u", ctx->cc_major, ctx->cc_minor,
                                ctx->sm_count, log2_bucket(n_scenes), log2_bucket(tris), log2_bucket(pixels),
                                p->max_depth);
    if (n < 0 || (uint32_t)n >= key_bytes) return rtc::set_error(ctx, RT_ERR_OOM, "rt_batch_tuning_key: key buffer too small");
    return RT_OK;
}

namespace {

struct Timer {
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Timer() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
    }
};

// Best of three graph launches after a warm-up; RT_OK and *ms, or an error.
int time_tuning(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n, const rt_batch_params *p,
                const rt_batch_tuning &t, void *scratch, uint64_t bytes, Timer &tm, float *ms) {
    rt_batch_plan *pl = nullptr;
    int rc = rt_batch_plan_create(ctx, scenes, n, p, &t, scratch, bytes, RT_BATCH_GRAPH | RT_BATCH_DISCARD, &pl);
    if (rc) return rc;
    float best = 0.0f;
    for (int it = 0; it < 4 && rc == RT_OK; ++it) {
        if (cudaEventRecord(tm.e0, tm.st) != cudaSuccess) rc = RT_ERR_CUDA;
        if (rc == RT_OK) rc = rt_batch_launch(pl, tm.st, 0u);
        if (rc == RT_OK && cudaEventRecord(tm.e1, tm.st) != cudaSuccess) rc = RT_ERR_CUDA;
        if (rc == RT_OK && cudaEventSynchronize(tm.e1) != cudaSuccess) rc = RT_ERR_CUDA;
        float x = 0.0f;
        if (rc == RT_OK && cudaEventElapsedTime(&x, tm.e0, tm.e1) != cudaSuccess) rc = RT_ERR_CUDA;
        if (rc == RT_OK && it > 0 && (it == 1 || x < best)) best = x;  // launch 0 warms up
    }
    rt_batch_plan_destroy(pl);
    if (rc == RT_OK) {
        uint32_t err[2] = {0u, 0u};
        if (cudaMemcpy(err, ctx->d_err, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess) return RT_ERR_CUDA;
        if (err[0]) return RT_ERR_BOUNDS;  // left on the device for rt_sync to report
    }
    *ms = best;
    return rc;
}

std::string describe(const rt_batch_tuning &t) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "threads %u, blocks/SM %u, ring %u, refill %u, shade %u, wave %u", t.trace_threads,
                  t.trace_blocks_per_sm, t.stack_ring, t.refill, t.shade_threads, t.wave_paths);
    return buf;
}

}  // namespace

extern "C" rt_status rt_batch_autotune(rt_context *ctx, const rt_batch_scene *scenes, uint32_t n_scenes,
                                       const rt_batch_params *p, void *scratch, uint64_t scratch_bytes,
                                       const char *cache_path, uint32_t flags, rt_batch_tuning *best,
                                       float *best_ms) {
    if (!ctx || !p || !best || (n_scenes && !scenes) || !scratch)
        return rtc::set_error(ctx, RT_ERR_INVALID_ARG, "rt_batch_autotune: null argument");
    if (flags & ~RT_TUNE_FORCE) return rtc::set_error(ctx, RT_ERR_INVALID_ARG, "rt_batch_autotune: unknown flags");
    char key[160];
    int rc = rt_batch_tuning_key(ctx, scenes, n_scenes, p, key, sizeof(key));
    if (rc) return rc;
    if (cache_path && !(flags & RT_TUNE_FORCE)) {
        float ms = 0.0f;
        rc = rt_batch_tuning_cache_lookup(cache_path, key, best, &ms);
        if (rc == RT_OK) {
            if (best_ms) *best_ms = ms;
            return RT_OK;
        }
        if (rc != RT_ERR_NOT_FOUND)
            return rtc::set_error(ctx, rc, "rt_batch_autotune: the cache file is not a readable tuning cache");
    }
    uint64_t need = 0;
    rc = rt_batch_scratch_bytes(scenes, n_scenes, p, nullptr, &need);
    if (rc) return rtc::set_error(ctx, rc, "rt_batch_autotune: invalid batch");
    if (scratch_bytes < need)
        return rtc::set_error(ctx, RT_ERR_OOM, "rt_batch_autotune: scratch smaller than rt_batch_scratch_bytes(NULL)");
    uint64_t paths = 0;
    for (uint32_t s = 0; s < n_scenes; ++s) paths += (uint64_t)scenes[s].width * scenes[s].height;

    rt_batch_params tp = *p;
    tp.spp = 1u;
    Timer tm;
    RT_CUDA_CTX(ctx, cudaSetDevice(ctx->device));
    RT_CUDA_CTX(ctx, cudaStreamCreateWithFlags(&tm.st, cudaStreamNonBlocking));
    RT_CUDA_CTX(ctx, cudaEventCreate(&tm.e0));
    RT_CUDA_CTX(ctx, cudaEventCreate(&tm.e1));

    Json trials;
    trials.kind = Json::Arr;
    auto record = [&](const rt_batch_tuning &t, float ms, bool ok) {
        Json e;
        e.kind = Json::Arr;
        e.arr.push_back(str(describe(t)));
        e.arr.push_back(ok ? num(std::round((double)ms * 1000.0) / 1000.0) : Json());
        trials.arr.push_back(e);
    };

    rt_batch_tuning cur;
    rt_batch_default_tuning(&cur);
    // the width the structures were built with (the first scene with pixels)
    for (uint32_t s = 0; s < n_scenes; ++s) {
        if (!((uint64_t)scenes[s].width * scenes[s].height) || !scenes[s].scene.accel) continue;
        uint32_t bf = 0;
        const void *src = reinterpret_cast<const uint8_t *>(scenes[s].scene.accel) + offsetof(rt_accel_header, build_flags);
        RT_CUDA_CTX(ctx, cudaMemcpy(&bf, src, sizeof(bf), cudaMemcpyDeviceToHost));
        const uint32_t w = (bf & RT_BUILD_WIDTH_MASK) >> 16;
        cur.bvh_width = w ? w : 8u;
        break;
    }
    float cur_ms = 0.0f;
    rc = time_tuning(ctx, scenes, n_scenes, &tp, cur, scratch, scratch_bytes, tm, &cur_ms);
    if (rc) return rc == RT_ERR_BOUNDS ? rc : rtc::set_error(ctx, rc, "rt_batch_autotune: the default tuning failed");
    record(cur, cur_ms, true);

    // coordinate descent; a candidate must beat the current best by 1 % (the
    // spread of repeated timings of one tuning is about that)
    auto tryit = [&](rt_batch_tuning cand) -> int {
        float ms = 0.0f;
        const int r = time_tuning(ctx, scenes, n_scenes, &tp, cand, scratch, scratch_bytes, tm, &ms);
        if (r == RT_ERR_BOUNDS || r == RT_ERR_CUDA) return r;  // a device fault is not a slow candidate
        record(cand, ms, r == RT_OK);
        if (r == RT_OK && ms < cur_ms * 0.99f) {
            cur = cand;
            cur_ms = ms;
        }
        return RT_OK;
    };
    // each list holds the values other than the default
    const uint32_t refills[] = {2u, 8u, 16u};
    const uint32_t rings[] = {8u, 32u};
    const uint32_t shades[] = {128u, 512u};
    for (uint32_t v : refills)
        if (v != cur.refill) {
            rt_batch_tuning c = cur;
            c.refill = v;
            if ((rc = tryit(c))) return rc;
        }
    for (uint32_t v : rings)
        if (v != cur.stack_ring) {
            rt_batch_tuning c = cur;
            c.stack_ring = v;
            if ((rc = tryit(c))) return rc;
        }
    {
        // the same threads per SM in blocks of 256
        rt_batch_tuning c = cur;
        c.trace_threads = cur.trace_threads == 128u ? 256u : 128u;
        c.trace_blocks_per_sm = cur.trace_threads == 128u ? (cur.trace_blocks_per_sm + 1u) / 2u
                                                          : cur.trace_blocks_per_sm * 2u;
        if ((rc = tryit(c))) return rc;
    }
    {
        const uint32_t full = 1024u / cur.trace_threads;  // 64-register kernels: 1024 threads per SM
        const uint32_t bps[] = {full / 2u, (full * 3u) / 4u, full};
        for (uint32_t v : bps)
            if (v && v != cur.trace_blocks_per_sm) {
                rt_batch_tuning c = cur;
                c.trace_blocks_per_sm = v;
                if ((rc = tryit(c))) return rc;
            }
    }
    for (uint32_t v : shades)
        if (v != cur.shade_threads) {
            rt_batch_tuning c = cur;
            c.shade_threads = v;
            if ((rc = tryit(c))) return rc;
        }
    for (uint32_t div : {2u, 4u}) {
        const uint64_t w = (paths / div + 1023u) / 1024u * 1024u;
        if (w >= 65536u && w < paths) {
            rt_batch_tuning c = cur;
            c.wave_paths = (uint32_t)w;
            if ((rc = tryit(c))) return rc;
        }
    }
    *best = cur;
    if (best_ms) *best_ms = cur_ms;
    if (cache_path) {
        rc = cache_store(cache_path, key, &cur, cur_ms, &trials);
        if (rc) return rtc::set_error(ctx, rc, "rt_batch_autotune: could not write the cache file");
    }
    return RT_OK;
}
