// ply.cu -- the scene file format: binary PLY vertex records <-> the
// per-primitive parameter tensors.
//
// The reference stores a scene as one PLY "vertex" element of float32
// properties x, y, z, red, green, blue, opacity, beta_*, mean_*, scale_*,
// l_triangle_* (scene/beta_model.py:286-320, written through plyfile as
// binary little-endian) and loads it back by property name
// (:322-404).  Here the header is parsed and the body read by host code of
// this library; the records travel to the device as they are and one kernel
// scatters their columns into the parameter tensors (or gathers them, to
// save), so no per-attribute host copies or float64 staging are made.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>

#include "ubs_common.cuh"

namespace ubs {
namespace {

struct PlyMap {
    int32_t A, n_tensors;
    int32_t unmapped; // some record property is filled by no tensor (packed as 0)
    int32_t w[UBS_PLY_MAX_TENSORS];
    int32_t off[UBS_PLY_MAX_TENSORS]; // first entry of each tensor in src_of
    float *p[UBS_PLY_MAX_TENSORS];
    int16_t tensor_of[UBS_PLY_MAX_PROPS];
    int16_t column_of[UBS_PLY_MAX_PROPS];
    int16_t src_of[UBS_PLY_MAX_PROPS];  // record column of each tensor column (-1: none)
};

constexpr int PLY_ROWS = 32; // records per warp step

// One warp per PLY_ROWS consecutive records: the records (contiguous) pass
// through shared memory, and each tensor's PLY_ROWS rows (contiguous in the
// tensor) are written -- or read, to pack -- as one run, so every global
// access is coalesced and no per-element division by the record width runs
// on 64-bit indices.
template <bool PACK>
__global__ void __launch_bounds__(256) ply_kernel(PlyMap m, float *records, int64_t n) {
    extern __shared__ float sbuf[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    float *sw = sbuf + (size_t)warp * PLY_ROWS * m.A;
    const int64_t groups = (n + PLY_ROWS - 1) / PLY_ROWS;
    for (int64_t gi = (int64_t)blockIdx.x * wpb + warp; gi < groups; gi += (int64_t)gridDim.x * wpb) {
        const int64_t r0 = gi * PLY_ROWS;
        const int rows = (int)(n - r0 < PLY_ROWS ? n - r0 : PLY_ROWS);
        const int cnt = rows * m.A;
        float *rec = records + r0 * m.A;
        if (!PACK) {
            for (int e = lane; e < cnt; e += 32) sw[e] = rec[e];
            __syncwarp();
            for (int k = 0; k < m.n_tensors; ++k) {
                const int w = m.w[k];
                float *dst = m.p[k] + r0 * w;
                for (int e = lane; e < rows * w; e += 32) {
                    const int r = e / w, c = e - r * w;
                    const int s = m.src_of[m.off[k] + c];
                    if (s >= 0) dst[e] = sw[r * m.A + s];
                }
            }
        } else {
            if (m.unmapped)
                for (int e = lane; e < cnt; e += 32) {
                    const int r = e / m.A, c = e - r * m.A;
                    if (m.tensor_of[c] < 0) sw[e] = 0.f; // properties no tensor fills
                }
            for (int k = 0; k < m.n_tensors; ++k) {
                const int w = m.w[k];
                const float *src = m.p[k] + r0 * w;
                for (int e = lane; e < rows * w; e += 32) {
                    const int r = e / w, c = e - r * w;
                    const int s = m.src_of[m.off[k] + c];
                    if (s >= 0) sw[r * m.A + s] = src[e];
                }
            }
            __syncwarp();
            for (int e = lane; e < cnt; e += 32) rec[e] = sw[e];
        }
        __syncwarp();
    }
}

int load_map(const ubs_ply_layout *l, PlyMap &m) {
    UBS_REQUIRE(l, "ply: null layout");
    UBS_REQUIRE(l->record_floats >= 1 && l->record_floats <= UBS_PLY_MAX_PROPS,
                "ply: 1..%d properties per vertex", UBS_PLY_MAX_PROPS);
    UBS_REQUIRE(l->n_tensors >= 0 && l->n_tensors <= UBS_PLY_MAX_TENSORS, "ply: bad tensor count");
    m.A = l->record_floats;
    m.n_tensors = l->n_tensors;
    for (int k = 0; k < UBS_PLY_MAX_TENSORS; ++k) {
        m.w[k] = k < l->n_tensors ? l->width[k] : 0;
        m.p[k] = k < l->n_tensors ? l->param[k] : nullptr;
        if (k < l->n_tensors) UBS_REQUIRE(m.p[k] && m.w[k] >= 1, "ply: bad tensor %d", k);
    }
    int total = 0;
    for (int k = 0; k < UBS_PLY_MAX_TENSORS; ++k) {
        m.off[k] = total;
        total += m.w[k];
    }
    UBS_REQUIRE(total <= UBS_PLY_MAX_PROPS, "ply: more than %d tensor columns", UBS_PLY_MAX_PROPS);
    for (int i = 0; i < UBS_PLY_MAX_PROPS; ++i) m.src_of[i] = -1;
    m.unmapped = 0;
    for (int c = 0; c < UBS_PLY_MAX_PROPS; ++c) {
        const bool in = c < m.A;
        m.tensor_of[c] = in ? l->tensor_of[c] : -1;
        m.column_of[c] = in ? l->column_of[c] : 0;
        if (in && m.tensor_of[c] >= 0) {
            UBS_REQUIRE(m.tensor_of[c] < m.n_tensors && m.column_of[c] >= 0 &&
                            m.column_of[c] < m.w[m.tensor_of[c]],
                        "ply: property %d maps outside its tensor", c);
            m.src_of[m.off[m.tensor_of[c]] + m.column_of[c]] = (int16_t)c;
        } else if (in) {
            m.unmapped = 1;
        }
    }
    return UBS_OK;
}

// Reads one header line (without its line break); false at end of file.
bool read_line(FILE *f, std::string &line) {
    line.clear();
    int ch;
    while ((ch = fgetc(f)) != EOF) {
        if (ch == '\n') return true;
        line.push_back((char)ch);
        if (line.size() > 4096) return false;
    }
    return !line.empty();
}

void strip_cr(std::string &s) {
    if (!s.empty() && s.back() == '\r') s.pop_back();
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

int ubs_ply_read_header(const char *path, int64_t *n_vertices, int32_t *n_props, char *names,
                        int32_t names_capacity, int64_t *body_offset) {
    UBS_REQUIRE(path && n_vertices && n_props && body_offset, "ply_read_header: null pointer");
    FILE *f = fopen(path, "rb");
    if (!f) return set_error(UBS_ERR_INVALID, "ply: cannot open %s: %s", path, strerror(errno));
    std::string line;
    int rc = UBS_OK;
    int64_t nv = -1;
    int32_t np = 0;
    bool in_vertex = false, ended = false;
    if (!read_line(f, line) || (strip_cr(line), line != "ply")) {
        rc = set_error(UBS_ERR_INVALID, "ply: %s is not a PLY file", path);
    }
    while (rc == UBS_OK && read_line(f, line)) {
        strip_cr(line);
        char w0[64] = {0}, w1[64] = {0}, w2[256] = {0};
        const int nw = sscanf(line.c_str(), "%63s %63s %255s", w0, w1, w2);
        if (nw <= 0) continue;
        if (!strcmp(w0, "end_header")) {
            ended = true;
            break;
        } else if (!strcmp(w0, "comment") || !strcmp(w0, "obj_info")) {
            continue;
        } else if (!strcmp(w0, "format")) {
            if (strcmp(w1, "binary_little_endian") != 0)
                rc = set_error(UBS_ERR_UNSUPPORTED,
                               "ply: format %s (only binary_little_endian is read)", w1);
        } else if (!strcmp(w0, "element")) {
            long long cnt = -1;
            if (nw < 3 || sscanf(w2, "%lld", &cnt) != 1 || cnt < 0) {
                rc = set_error(UBS_ERR_INVALID, "ply: bad element line '%s'", line.c_str());
            } else if (!strcmp(w1, "vertex")) {
                if (nv >= 0) rc = set_error(UBS_ERR_INVALID, "ply: two vertex elements");
                nv = cnt;
                in_vertex = true;
            } else {
                in_vertex = false;
                if (nv < 0 || cnt > 0)
                    rc = set_error(UBS_ERR_UNSUPPORTED,
                                   "ply: element '%s' besides the vertices is not read", w1);
            }
        } else if (!strcmp(w0, "property")) {
            if (!in_vertex) {
                continue; // a property of an empty element after the vertices
            }
            if (strcmp(w1, "float") != 0 && strcmp(w1, "float32") != 0) {
                rc = set_error(UBS_ERR_UNSUPPORTED,
                               "ply: vertex property '%s' of type %s (only float is read)", w2,
                               w1);
            } else if (np >= UBS_PLY_MAX_PROPS) {
                rc = set_error(UBS_ERR_UNSUPPORTED, "ply: more than %d vertex properties",
                               UBS_PLY_MAX_PROPS);
            } else {
                if (names && np < names_capacity) {
                    strncpy(names + (size_t)np * UBS_PLY_NAME_BYTES, w2, UBS_PLY_NAME_BYTES - 1);
                    names[(size_t)np * UBS_PLY_NAME_BYTES + UBS_PLY_NAME_BYTES - 1] = 0;
                }
                ++np;
            }
        } else {
            rc = set_error(UBS_ERR_INVALID, "ply: unexpected header line '%s'", line.c_str());
        }
    }
    if (rc == UBS_OK && (!ended || nv < 0))
        rc = set_error(UBS_ERR_INVALID, "ply: %s has no complete header with vertices", path);
    if (rc == UBS_OK) {
        const long long off = ftell(f);
        fseek(f, 0, SEEK_END);
        const long long size = ftell(f);
        if (size - off < nv * (long long)np * 4)
            rc = set_error(UBS_ERR_INVALID, "ply: %s is truncated (%lld of %lld body bytes)",
                           path, size - off, nv * (long long)np * 4);
        *n_vertices = nv;
        *n_props = np;
        *body_offset = off;
    }
    fclose(f);
    return rc;
}

int ubs_ply_read_body(const char *path, int64_t offset, void *dst, int64_t n_bytes) {
    UBS_REQUIRE(path && (dst || n_bytes == 0) && offset >= 0 && n_bytes >= 0,
                "ply_read_body: bad arguments");
    FILE *f = fopen(path, "rb");
    if (!f) return set_error(UBS_ERR_INVALID, "ply: cannot open %s: %s", path, strerror(errno));
    int rc = UBS_OK;
    if (fseek(f, (long)offset, SEEK_SET) != 0 ||
        fread(dst, 1, (size_t)n_bytes, f) != (size_t)n_bytes)
        rc = set_error(UBS_ERR_INVALID, "ply: short read from %s", path);
    fclose(f);
    return rc;
}

int ubs_ply_write(const char *path, int64_t n_vertices, int32_t n_props, const char *names,
                  const void *records) {
    UBS_REQUIRE(path && names && n_vertices >= 0 && n_props >= 1 &&
                    (records || n_vertices == 0),
                "ply_write: bad arguments");
    FILE *f = fopen(path, "wb");
    if (!f) return set_error(UBS_ERR_INVALID, "ply: cannot create %s: %s", path, strerror(errno));
    int rc = UBS_OK;
    std::string h = "ply\nformat binary_little_endian 1.0\nelement vertex " +
                    std::to_string((long long)n_vertices) + "\n";
    for (int i = 0; i < n_props; ++i) {
        const char *nm = names + (size_t)i * UBS_PLY_NAME_BYTES;
        h += "property float ";
        h.append(nm, strnlen(nm, UBS_PLY_NAME_BYTES));
        h += "\n";
    }
    h += "end_header\n";
    const size_t body = (size_t)n_vertices * n_props * 4;
    if (fwrite(h.data(), 1, h.size(), f) != h.size() ||
        (body && fwrite(records, 1, body, f) != body))
        rc = set_error(UBS_ERR_INVALID, "ply: short write to %s", path);
    if (fclose(f) != 0 && rc == UBS_OK) rc = set_error(UBS_ERR_INVALID, "ply: close failed");
    return rc;
}

static int ply_launch(const ubs_ply_layout *layout, float *records, int64_t n, void *stream,
                      bool pack) {
    UBS_REQUIRE(n >= 0 && (records || n == 0), "ply: bad records");
    if (n == 0) return UBS_OK; // nothing to move (empty tensors have no storage)
    PlyMap m;
    const int rc = load_map(layout, m);
    if (rc != UBS_OK) return rc;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // warps per block by the shared memory one warp's records take (<= 48 KB)
    const size_t per_warp = (size_t)PLY_ROWS * m.A * sizeof(float);
    int wpb = (int)((48 * 1024) / per_warp);
    wpb = wpb < 1 ? 1 : (wpb > 8 ? 8 : wpb);
    const int64_t groups = (n + PLY_ROWS - 1) / PLY_ROWS;
    const int64_t want = (groups + wpb - 1) / wpb;
    const unsigned grid = (unsigned)(want < (int64_t)sms * 16 ? want : (int64_t)sms * 16);
    const size_t smem = per_warp * wpb;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (pack)
        UBS_TIMED("ply_pack", st, ply_kernel<true><<<grid, 32 * wpb, smem, st>>>(m, records, n));
    else
        UBS_TIMED("ply_unpack", st, ply_kernel<false><<<grid, 32 * wpb, smem, st>>>(m, records, n));
    note_launch();
    return check_launch(pack ? "ply_pack" : "ply_unpack");
}

int ubs_ply_unpack(const ubs_ply_layout *layout, const float *records, int64_t n_vertices,
                   void *stream) {
    return ply_launch(layout, const_cast<float *>(records), n_vertices, stream, false);
}

int ubs_ply_pack(const ubs_ply_layout *layout, float *records, int64_t n_vertices,
                 void *stream) {
    return ply_launch(layout, records, n_vertices, stream, true);
}

} // extern "C"
