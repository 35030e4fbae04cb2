// bg_io.cpp - scene and film I/O around the render path: Wavefront OBJ triangle meshes in, the
// resolved film out as OpenEXR.
//
// OBJ follows OBJ::read (src/io/obj.rs:16-123): a line starting with 'f' appends one vertex index
// per token (forms "v", "v/vt", "v/vt/vn", "v//vn"; 1-based), a line starting with "vt" / "vn" /
// 'v' appends a texture coordinate / normal / position (the first three values), and the mesh is
// the consecutive triples of all face indices in file order (polygons with more than three
// corners are not fanned; a trailing partial triple is dropped).  Positions go through the
// object-to-world transform and normals through its inverse transpose (TriangleMesh::new,
// src/shapes/triangle.rs:48-90; both skipped for the identity).  The i-th face vertex takes the
// i-th normal index and the i-th texture index of the file, as the reference pairs them; a mesh
// has per-vertex normals / uvs when any face gives them.  The mesh's triangles swap handedness
// when the inverse transform has a negative determinant (Triangle::new, triangle.rs:94-105).
// Where the reference panics (unreadable file, bad number, index 0 or past the end, a 'v' line
// with fewer than three values, fewer normal or texture indices than face vertices) this returns
// BG_ERR_INVALID with the line number.
//
// EXR: a single-part scanline file, uncompressed, channels B G R as 32-bit float, one scanline per
// block - what Image::write (src/io/image.rs:47-53) stores for an Rgb32F buffer, headless.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bonsai_gpu.h"
#include "bg_internal.h"

namespace {

void set_err(char* buf, size_t len, const std::string& msg) {
    if (buf && len) {
        std::strncpy(buf, msg.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
}

bool parse_index(const std::string& tok, size_t* out) {  // Rust `usize::from_str`
    if (tok.empty()) return false;
    size_t i = tok[0] == '+' ? 1 : 0;
    if (i == tok.size()) return false;
    uint64_t v = 0;
    for (; i < tok.size(); ++i) {
        if (tok[i] < '0' || tok[i] > '9') return false;
        uint64_t nv = v * 10 + (uint64_t)(tok[i] - '0');
        if (nv / 10 != v) return false;
        v = nv;
    }
    *out = (size_t)v;
    return true;
}

bool parse_float(const std::string& tok, float* out) {  // Rust `f32::from_str` (decimal / exponent / inf / nan)
    if (tok.empty()) return false;
    const char* s = tok.c_str();
    char* end = nullptr;
    errno = 0;
    float v = std::strtof(s, &end);
    if (end != s + tok.size()) return false;
    if (tok.find_first_of("xXpP") != std::string::npos) return false;  // no hex floats
    *out = v;
    return true;
}

std::vector<std::string> split_ws(const std::string& line) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && std::isspace((unsigned char)line[i])) ++i;
        size_t j = i;
        while (j < line.size() && !std::isspace((unsigned char)line[j])) ++j;
        if (j > i) out.push_back(line.substr(i, j - i));
        i = j;
    }
    return out;
}

std::vector<std::string> split_on(const std::string& s, const std::string& sep) {
    std::vector<std::string> out;
    size_t i = 0;
    for (;;) {
        size_t j = s.find(sep, i);
        if (j == std::string::npos) {
            out.push_back(s.substr(i));
            return out;
        }
        out.push_back(s.substr(i, j - i));
        i = j + sep.size();
    }
}

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

struct ObjMesh {
    std::vector<float> tri;  // 9 per triangle, world space
    std::vector<float> nrm;  // 9 per triangle, or empty
    std::vector<float> uv;   // 6 per triangle, or empty
    uint32_t flags = 0;      // BG_TRI_SWAPS_HANDEDNESS
};

bool is_identity(const float* xf) {
    if (!xf) return true;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c)
            if (xf[4 * r + c] != (r == c ? 1.0f : 0.0f)) return false;
    return true;
}

// Parses the file into world-space triangles, with their vertex normals and uvs when `attrs`.
bool read_obj(const char* path, const float* xf, ObjMesh* mesh, std::string* err, bool attrs = true) {
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        *err = std::string("cannot open ") + path;
        return false;
    }
    std::vector<float> pos, nrm, uvv;
    std::vector<size_t> vi, ni, ti;
    std::vector<size_t> vi_line;  // line of each face index, for messages
    std::string line;
    size_t lineno = 0;
    char buf[4096];
    bool ok = true;
    auto fail = [&](const std::string& m) {
        *err = std::string(path) + ":" + std::to_string(lineno) + ": " + m;
        ok = false;
    };
    while (ok) {
        line.clear();
        bool got = false;
        while (std::fgets(buf, sizeof(buf), f)) {
            got = true;
            line += buf;
            if (!line.empty() && line.back() == '\n') break;
        }
        if (!got) break;
        ++lineno;
        const std::string t = trim(line);
        if (!t.empty() && t[0] == 'f') {
            std::vector<std::string> toks = split_ws(t);
            for (size_t k = 1; k < toks.size() && ok; ++k) {
                const std::string& v = toks[k];
                size_t a = 0, b = 0, c = 0;
                if (v.find("//") != std::string::npos) {
                    std::vector<std::string> p = split_on(v, "//");
                    if (p.size() != 2 || !parse_index(p[0], &a) || !parse_index(p[1], &b)) fail("bad face token " + v);
                    else {
                        vi.push_back(a);
                        ni.push_back(b);
                    }
                } else if (v.find('/') != std::string::npos) {
                    std::vector<std::string> p = split_on(v, "/");
                    if ((p.size() != 2 && p.size() != 3) || !parse_index(p[0], &a) || !parse_index(p[1], &b) ||
                        (p.size() == 3 && !parse_index(p[2], &c)))
                        fail("bad face token " + v);
                    else {
                        vi.push_back(a);
                        ti.push_back(b);
                        if (p.size() == 3) ni.push_back(c);
                    }
                } else if (!parse_index(v, &a)) {
                    fail("bad face index " + v);
                } else {
                    vi.push_back(a);
                }
                vi_line.push_back(lineno);
            }
        }
        if (ok && !t.empty() && t[0] == 'v') {
            std::vector<std::string> toks = split_ws(t);
            std::vector<float> p;
            for (size_t k = 1; k < toks.size() && ok; ++k) {
                float x;
                if (!parse_float(toks[k], &x)) fail("bad number " + toks[k]);
                else p.push_back(x);
            }
            if (!ok) break;
            if (t.rfind("vt", 0) == 0) {
                if (p.size() < 2) fail("texture coordinate needs 2 values");
                else uvv.insert(uvv.end(), p.begin(), p.begin() + 2);
            } else if (t.rfind("vn", 0) == 0) {
                if (p.size() < 3) fail("normal needs 3 values");
                else nrm.insert(nrm.end(), p.begin(), p.begin() + 3);
            } else {
                if (p.size() < 3) fail("position needs 3 values");
                else pos.insert(pos.end(), p.begin(), p.begin() + 3);
            }
        }
    }
    std::fclose(f);
    if (!ok) return false;
    const size_t npos = pos.size() / 3, nnormals = nrm.size() / 3, nuvs = uvv.size() / 2;
    for (size_t i = 0; i < vi.size(); ++i)
        if (vi[i] == 0 || vi[i] > npos) {
            *err = std::string(path) + ":" + std::to_string(vi_line[i]) + ": position index " + std::to_string(vi[i]) +
                   " out of range";
            return false;
        }
    for (size_t i = 0; i < ni.size(); ++i)
        if (ni[i] == 0 || ni[i] > nnormals) {
            *err = std::string(path) + ": normal index " + std::to_string(ni[i]) + " out of range";
            return false;
        }
    for (size_t i = 0; i < ti.size(); ++i)
        if (ti[i] == 0 || ti[i] > nuvs) {
            *err = std::string(path) + ": texture index " + std::to_string(ti[i]) + " out of range";
            return false;
        }
    const size_t ntri = vi.size() / 3;
    if (!attrs) {
        ni.clear();
        ti.clear();
    }
    // a triangle reads normal[3t + k] / uv[3t + k]: the lists must cover every used face vertex
    if (!ni.empty() && ni.size() < 3 * ntri) {
        *err = std::string(path) + ": " + std::to_string(ni.size()) + " normal indices for " +
               std::to_string(3 * ntri) + " triangle vertices";
        return false;
    }
    if (!ti.empty() && ti.size() < 3 * ntri) {
        *err = std::string(path) + ": " + std::to_string(ti.size()) + " texture indices for " +
               std::to_string(3 * ntri) + " triangle vertices";
        return false;
    }
    const bool ident = is_identity(xf);
    float inv[12];
    if (!ident) {
        bgi::affine_inverse(xf, inv);
        // Transform::swaps_handedness of world_to_object = the inverse (transform.rs:218-224)
        float det = inv[0] * (inv[5] * inv[10] - inv[6] * inv[9]) - inv[1] * (inv[4] * inv[10] - inv[6] * inv[8]) +
                    inv[2] * (inv[4] * inv[9] - inv[5] * inv[8]);
        if (det < 0.0f) mesh->flags |= BG_TRI_SWAPS_HANDEDNESS;
    }
    mesh->tri.resize(ntri * 9);
    if (!ni.empty()) mesh->nrm.resize(ntri * 9);
    if (!ti.empty()) mesh->uv.resize(ntri * 6);
    for (size_t k = 0; k < ntri * 3; ++k) {
        const float* p = &pos[3 * (vi[k] - 1)];
        float* o = &mesh->tri[3 * k];
        if (!ident) {  // Point3::transform of an affine matrix (w = 1)
            for (int r = 0; r < 3; ++r)
                o[r] = xf[4 * r] * p[0] + xf[4 * r + 1] * p[1] + xf[4 * r + 2] * p[2] + xf[4 * r + 3];
        } else {
            o[0] = p[0];
            o[1] = p[1];
            o[2] = p[2];
        }
        if (!ni.empty()) {
            const float* n = &nrm[3 * (ni[k] - 1)];
            float* q = &mesh->nrm[3 * k];
            if (!ident) {  // Normal::transform: m_inverse transposed (normal.rs:21-30)
                for (int c = 0; c < 3; ++c) q[c] = inv[c] * n[0] + inv[4 + c] * n[1] + inv[8 + c] * n[2];
            } else {
                q[0] = n[0];
                q[1] = n[1];
                q[2] = n[2];
            }
        }
        if (!ti.empty()) {
            mesh->uv[2 * k] = uvv[2 * (ti[k] - 1)];
            mesh->uv[2 * k + 1] = uvv[2 * (ti[k] - 1) + 1];
        }
    }
    return true;
}

void put32(std::vector<uint8_t>& b, uint32_t v) {
    for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
    for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void putf(std::vector<uint8_t>& b, float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    put32(b, u);
}
void put_str(std::vector<uint8_t>& b, const char* s) { b.insert(b.end(), s, s + std::strlen(s) + 1); }
void attr(std::vector<uint8_t>& b, const char* name, const char* type, const std::vector<uint8_t>& v) {
    put_str(b, name);
    put_str(b, type);
    put32(b, (uint32_t)v.size());
    b.insert(b.end(), v.begin(), v.end());
}

bool write_exr(const char* path, const float* rgb, uint32_t w, uint32_t h, std::string* err) {
    std::vector<uint8_t> b;
    put32(b, 20000630u);  // magic 76 2f 31 01
    put32(b, 2u);         // version 2, single-part scanline
    std::vector<uint8_t> ch;
    for (const char* c : {"B", "G", "R"}) {  // alphabetical
        put_str(ch, c);
        put32(ch, 2u);  // FLOAT
        ch.push_back(0);  // pLinear
        ch.push_back(0);
        ch.push_back(0);
        ch.push_back(0);
        put32(ch, 1u);  // xSampling
        put32(ch, 1u);  // ySampling
    }
    ch.push_back(0);
    attr(b, "channels", "chlist", ch);
    attr(b, "compression", "compression", {0});
    std::vector<uint8_t> box;
    put32(box, 0);
    put32(box, 0);
    put32(box, w - 1);
    put32(box, h - 1);
    attr(b, "dataWindow", "box2i", box);
    attr(b, "displayWindow", "box2i", box);
    attr(b, "lineOrder", "lineOrder", {0});
    std::vector<uint8_t> one;
    putf(one, 1.0f);
    attr(b, "pixelAspectRatio", "float", one);
    std::vector<uint8_t> c2;
    putf(c2, 0.0f);
    putf(c2, 0.0f);
    attr(b, "screenWindowCenter", "v2f", c2);
    attr(b, "screenWindowWidth", "float", one);
    b.push_back(0);  // end of header
    const uint64_t line_bytes = 8 + (uint64_t)w * 3 * 4;
    const uint64_t table_end = b.size() + 8ull * h;
    for (uint32_t y = 0; y < h; ++y) put64(b, table_end + y * line_bytes);
    for (uint32_t y = 0; y < h; ++y) {
        put32(b, y);
        put32(b, w * 3 * 4);
        for (int c = 2; c >= 0; --c)  // B, G, R planes of the scanline
            for (uint32_t x = 0; x < w; ++x) putf(b, rgb[3 * ((size_t)y * w + x) + c]);
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        *err = std::string("cannot create ") + path;
        return false;
    }
    bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) *err = std::string("write failed: ") + path;
    return ok;
}

}  // namespace

extern "C" {

bg_status bg_obj_read(const char* path, const float* object_to_world, float* tri_out, size_t max_tri, size_t* ntri,
                      char* err, size_t err_len) {
    if (!path || !ntri || (max_tri && !tri_out)) return BG_ERR_INVALID;
    ObjMesh m;
    std::string msg;
    if (!read_obj(path, object_to_world, &m, &msg, false)) {
        set_err(err, err_len, msg);
        return BG_ERR_INVALID;
    }
    *ntri = m.tri.size() / 9;
    if (tri_out) std::memcpy(tri_out, m.tri.data(), std::min(max_tri, *ntri) * 9 * sizeof(float));
    return BG_OK;
}

bg_status bg_obj_read_mesh(const char* path, const float* object_to_world, float* tri_out, float* normal_out,
                           float* uv_out, size_t max_tri, bg_obj_info* info, char* err, size_t err_len) {
    if (!path || !info || (max_tri && !tri_out)) return BG_ERR_INVALID;
    ObjMesh m;
    std::string msg;
    if (!read_obj(path, object_to_world, &m, &msg)) {
        set_err(err, err_len, msg);
        return BG_ERR_INVALID;
    }
    const size_t n = m.tri.size() / 9, k = std::min(max_tri, n);
    info->ntri = n;
    info->has_normals = m.nrm.empty() ? 0u : 1u;
    info->has_uvs = m.uv.empty() ? 0u : 1u;
    info->flags = m.flags;
    if (tri_out) std::memcpy(tri_out, m.tri.data(), k * 9 * sizeof(float));
    if (normal_out && !m.nrm.empty()) std::memcpy(normal_out, m.nrm.data(), k * 9 * sizeof(float));
    if (uv_out && !m.uv.empty()) std::memcpy(uv_out, m.uv.data(), k * 6 * sizeof(float));
    return BG_OK;
}

bg_status bg_scene_add_obj(bg_scene* s, const char* path, const float* object_to_world, uint32_t material_id,
                           int32_t light_id, size_t* ntri) {
    if (!s || !path) return BG_ERR_INVALID;
    if (!s->ctx) return BG_ERR_INVALID;
    ObjMesh m;
    std::string msg;
    if (!read_obj(path, object_to_world, &m, &msg)) return bgi::fail(s->ctx, BG_ERR_INVALID, msg);
    const size_t n = m.tri.size() / 9;
    std::vector<uint32_t> mat(n, material_id);
    std::vector<int32_t> light(n, light_id);
    bg_status st = bg_scene_add_triangle_mesh(s, m.tri.data(), n, mat.data(), light.data(),
                                              m.nrm.empty() ? nullptr : m.nrm.data(),
                                              m.uv.empty() ? nullptr : m.uv.data(), m.flags);
    if (st == BG_OK && ntri) *ntri = n;
    return st;
}

bg_status bg_write_exr(const char* path, const float* rgb, uint32_t width, uint32_t height) {
    if (!path || !rgb || width == 0 || height == 0) return BG_ERR_INVALID;
    std::string msg;
    return write_exr(path, rgb, width, height, &msg) ? BG_OK : BG_ERR_INVALID;
}

bg_status bg_film_write_exr(bg_ctx* ctx, const char* path) {
    if (!ctx || !path) return BG_ERR_INVALID;
    if (!ctx->film.rgb) return bgi::fail(ctx, BG_ERR_INVALID, "no film rendered yet");
    std::vector<float> rgb((size_t)ctx->film.npix * 3);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rgb.data(), ctx->film.rgb, rgb.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return bgi::cuda_fail(ctx, e, "film read-back");
    std::string msg;
    if (!write_exr(path, rgb.data(), ctx->film_w, ctx->film_h, &msg)) return bgi::fail(ctx, BG_ERR_INVALID, msg);
    return BG_OK;
}

}  // extern "C"
