// rt_io.cpp -- scene ingestion on the host: Wavefront OBJ meshes and
// Radiance RGBE (.hdr) environment maps.
//
// Follows the reference loader's rules (io/ObjLoader.cpp:97-290), so that a
// mesh read here has the vertices, normals, UVs and triangle order the
// reference's MeshFactory builds (factory/MeshFactory.h:39-139):
//   * "v" positions and "vn" normals are transformed by toWorld when read
//     (points with the homogeneous divide of Transform::transform(Point3d),
//     core/Transform.h:90-99; normals by the transposed inverse,
//     core/Transform.h:176-183); "vt" coordinates are kept as read;
//   * a face corner "p", "p/t", "p//n" or "p/t/n" is one vertex; a corner
//     without a UV or normal index refers to the first UV / normal; negative
//     indices count back from the end of the whole file's list (the reference
//     resolves them after reading, not at the face as the OBJ format says);
//   * corners are de-duplicated by their (p, t, n) triple in order of first
//     use, and the mesh's vertex arrays are built in that order;
//   * a face "a b c" is one triangle; "a b c d" is two, (a b c) and (d a c);
//     corners past the fourth are ignored, as in the reference;
//   * materials (useMtl / usemtl / mtllib) are not read: the BSDF comes from
//     the scene description.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "rt_internal.h"

namespace {

struct Corner {
    int p = 0, t = 1, n = 1;
    bool operator==(const Corner &o) const { return p == o.p && t == o.t && n == o.n; }
};
struct CornerHash {
    size_t operator()(const Corner &c) const
    {
        uint64_t h = (uint32_t)c.p;
        h = h * 0x9E3779B97F4A7C15ull ^ (uint32_t)c.t;
        h = h * 0x9E3779B97F4A7C15ull ^ (uint32_t)c.n;
        return (size_t)(h ^ (h >> 29));
    }
};

// "p[/[t][/n]]" -> corner; false on malformed input
bool parse_corner(const char *s, const char *e, Corner &c)
{
    c = Corner();
    c.t = 1;
    c.n = 1;
    const char *q = s;
    char *end = nullptr;
    long v = std::strtol(q, &end, 10);
    if (end == q) return false;
    c.p = (int)v;
    q = end;
    if (q < e && *q == '/') {
        q++;
        if (q < e && *q != '/') {
            v = std::strtol(q, &end, 10);
            if (end == q) return false;
            c.t = (int)v;
            q = end;
        }
        if (q < e && *q == '/') {
            q++;
            if (q < e) {
                v = std::strtol(q, &end, 10);
                if (end == q) return false;
                c.n = (int)v;
                q = end;
            }
        }
    }
    return q == e;
}

const char *skip_ws(const char *p, const char *e)
{
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
    return p;
}
const char *token_end(const char *p, const char *e)
{
    while (p < e && *p != ' ' && *p != '\t' && *p != '\r') p++;
    return p;
}

// binary32 values as the reference's stream extraction into `real` (float)
// reads them (correctly rounded); missing values stay 0
int read_floats(const char *p, const char *e, float *out, int n)
{
    int k = 0;
    while (k < n) {
        p = skip_ws(p, e);
        if (p >= e) break;
        char *end = nullptr;
        float v = std::strtof(p, &end);
        if (end == p) break;
        out[k++] = v;
        p = end;
    }
    return k;
}

}  // namespace

extern "C" rt_status rt_obj_load(const char *path, const float *to_world, rt_mesh_data *out)
{
    if (!path || !out) return rt_internal_error(RT_ERR_INVALID, "rt_obj_load: null argument");
    std::memset(out, 0, sizeof(*out));
    FILE *f = std::fopen(path, "rb");
    if (!f) return rt_internal_error(RT_ERR_INVALID, (std::string("rt_obj_load: cannot open ") + path).c_str());
    std::string text;
    {
        std::fseek(f, 0, SEEK_END);
        long sz = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (sz > 0) {
            text.resize((size_t)sz);
            if (std::fread(&text[0], 1, (size_t)sz, f) != (size_t)sz) {
                std::fclose(f);
                return rt_internal_error(RT_ERR_INVALID, "rt_obj_load: read failed");
            }
        }
        std::fclose(f);
    }
    // toWorld in binary32, row-major, applied as Transform::transform does
    // (operation order kept; the file is compiled without contraction)
    float M[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    if (to_world)
        for (int i = 0; i < 16; i++) M[i] = to_world[i];
    // transposed inverse of the upper 3x3 for normals (inverted in double;
    // the reference inverts the 4x4 with Eigen, equal for affine matrices up
    // to rounding)
    double a = M[0], b = M[1], c = M[2], d = M[4], e = M[5], g = M[6], h = M[8], i3 = M[9], k = M[10];
    double det = a * (e * k - g * i3) - b * (d * k - g * h) + c * (d * i3 - e * h);
    float NI[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (det != 0.0) {
        double inv[9] = {(e * k - g * i3) / det, (c * i3 - b * k) / det, (b * g - c * e) / det,
                         (g * h - d * k) / det, (a * k - c * h) / det, (c * d - a * g) / det,
                         (d * i3 - e * h) / det, (b * h - a * i3) / det, (a * e - b * d) / det};
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) NI[3 * r + q] = (float)inv[3 * q + r];
    }
    std::vector<float> P, N, T;
    std::vector<Corner> corners;
    std::vector<int> idx;
    std::unordered_map<Corner, int, CornerHash> cmap;
    const char *s = text.data(), *end = s + text.size();
    int line_no = 0;
    while (s < end) {
        const char *le = (const char *)std::memchr(s, '\n', (size_t)(end - s));
        if (!le) le = end;
        line_no++;
        const char *p = skip_ws(s, le);
        const char *te = token_end(p, le);
        size_t tl = (size_t)(te - p);
        if (tl == 1 && p[0] == 'v') {
            float v[3] = {0, 0, 0};
            read_floats(te, le, v, 3);
            float x = M[0] * v[0] + M[1] * v[1] + M[2] * v[2] + M[3];
            float y = M[4] * v[0] + M[5] * v[1] + M[6] * v[2] + M[7];
            float z = M[8] * v[0] + M[9] * v[1] + M[10] * v[2] + M[11];
            float w = M[12] * v[0] + M[13] * v[1] + M[14] * v[2] + M[15];
            if (w != 1.f && w != 0.f) { x /= w; y /= w; z /= w; }
            P.push_back(x); P.push_back(y); P.push_back(z);
        } else if (tl == 2 && p[0] == 'v' && p[1] == 'n') {
            float v[3] = {0, 0, 0};
            read_floats(te, le, v, 3);
            for (int r = 0; r < 3; r++) N.push_back(NI[3 * r] * v[0] + NI[3 * r + 1] * v[1] + NI[3 * r + 2] * v[2]);
        } else if (tl == 2 && p[0] == 'v' && p[1] == 't') {
            float v[2] = {0, 0};
            read_floats(te, le, v, 2);
            T.push_back(v[0]); T.push_back(v[1]);
        } else if (tl == 1 && p[0] == 'f') {
            Corner cs[4];
            int nc = 0;
            const char *q = te;
            while (nc < 5) {
                q = skip_ws(q, le);
                if (q >= le) break;
                const char *qe = token_end(q, le);
                if (nc < 4) {
                    if (!parse_corner(q, qe, cs[nc]))
                        return rt_internal_error(RT_ERR_INVALID,
                                                 ("rt_obj_load: bad face corner on line " + std::to_string(line_no)).c_str());
                }
                nc++;
                q = qe;
            }
            if (nc < 3)
                return rt_internal_error(RT_ERR_INVALID,
                                         ("rt_obj_load: face with fewer than 3 corners on line " + std::to_string(line_no)).c_str());
            Corner tri[6] = {cs[0], cs[1], cs[2], cs[0], cs[0], cs[0]};
            int nv = 3;
            if (nc >= 4) { tri[3] = cs[3]; tri[4] = cs[0]; tri[5] = cs[2]; nv = 6; }
            for (int t = 0; t < nv; t++) {
                auto it = cmap.find(tri[t]);
                if (it == cmap.end()) {
                    int id = (int)corners.size();
                    cmap.emplace(tri[t], id);
                    corners.push_back(tri[t]);
                    idx.push_back(id);
                } else {
                    idx.push_back(it->second);
                }
            }
        }
        s = le + 1;
    }
    const int nv = (int)corners.size();
    const int np = (int)P.size() / 3, nn = (int)N.size() / 3, nt = (int)T.size() / 2;
    auto resolve = [](int i, int n) { return i < 0 ? n + i + 1 : i; };
    std::vector<float> V(3 * (size_t)nv), VN, VT;
    for (int v = 0; v < nv; v++) {
        int pi = resolve(corners[v].p, np) - 1;
        if (pi < 0 || pi >= np) return rt_internal_error(RT_ERR_INVALID, "rt_obj_load: position index out of range");
        for (int q = 0; q < 3; q++) V[3 * (size_t)v + q] = P[3 * (size_t)pi + q];
    }
    if (nn > 0) {
        VN.resize(3 * (size_t)nv);
        for (int v = 0; v < nv; v++) {
            int ni = resolve(corners[v].n, nn) - 1;
            if (ni < 0 || ni >= nn) return rt_internal_error(RT_ERR_INVALID, "rt_obj_load: normal index out of range");
            for (int q = 0; q < 3; q++) VN[3 * (size_t)v + q] = N[3 * (size_t)ni + q];
        }
    }
    if (nt > 0) {
        VT.resize(2 * (size_t)nv);
        for (int v = 0; v < nv; v++) {
            int ti = resolve(corners[v].t, nt) - 1;
            if (ti < 0 || ti >= nt) return rt_internal_error(RT_ERR_INVALID, "rt_obj_load: uv index out of range");
            VT[2 * (size_t)v] = T[2 * (size_t)ti];
            VT[2 * (size_t)v + 1] = T[2 * (size_t)ti + 1];
        }
    }
    auto dup = [](const std::vector<float> &x) -> float * {
        if (x.empty()) return nullptr;
        float *p = (float *)std::malloc(x.size() * sizeof(float));
        if (p) std::memcpy(p, x.data(), x.size() * sizeof(float));
        return p;
    };
    out->n_vertices = nv;
    out->n_triangles = (int32_t)(idx.size() / 3);
    out->vertices = dup(V);
    out->normals = dup(VN);
    out->uvs = dup(VT);
    out->indices = idx.empty() ? nullptr : (int32_t *)std::malloc(idx.size() * sizeof(int32_t));
    if (out->indices) std::memcpy(out->indices, idx.data(), idx.size() * sizeof(int32_t));
    if ((nv && !out->vertices) || (!idx.empty() && !out->indices) || (!VN.empty() && !out->normals) ||
        (!VT.empty() && !out->uvs)) {
        rt_mesh_data_free(out);
        return rt_internal_error(RT_ERR_NOMEM, "rt_obj_load: out of host memory");
    }
    return RT_OK;
}

extern "C" void rt_mesh_data_free(rt_mesh_data *m)
{
    if (!m) return;
    std::free(m->vertices);
    std::free(m->normals);
    std::free(m->uvs);
    std::free(m->indices);
    std::memset(m, 0, sizeof(*m));
}

// ---------------------------------------------------------------------------
// Radiance RGBE images, as the reference reads environment maps: stb_image's
// stbi_loadf (io/ImageLoader.cpp:78-99; stb_image is not in the reference
// tree).  The published format: a "#?RADIANCE" or "#?RGBE" header with a
// FORMAT=32-bit_rle_rgbe line, a blank line, a "-Y height +X width"
// resolution line, then one scanline per row from the top, each either flat
// RGBE pixels or (for widths 8..32767) the adaptive run-length form: the
// marker 2 2 w>>8 w&255, then the four channels one after another, each as
// runs (count > 128: count - 128 copies of the next byte) and literals.
// A pixel (r, g, b, e) decodes as c * 2^(e - 136), or 0 when e == 0 (stb's
// conversion).  Rows are returned top first, RGB floats, row-major.
extern "C" rt_status rt_hdr_load(const char *path, int32_t *width, int32_t *height, float **rgb)
{
    if (!path || !width || !height || !rgb) return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: null argument");
    *rgb = nullptr;
    *width = *height = 0;
    FILE *f = std::fopen(path, "rb");
    if (!f) return rt_internal_error(RT_ERR_INVALID, (std::string("rt_hdr_load: cannot open ") + path).c_str());
    std::vector<unsigned char> buf;
    {
        std::fseek(f, 0, SEEK_END);
        long sz = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (sz > 0) {
            buf.resize((size_t)sz);
            if (std::fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) buf.clear();
        }
        std::fclose(f);
    }
    size_t pos = 0;
    auto line = [&](std::string &out) -> bool {
        out.clear();
        if (pos >= buf.size()) return false;
        while (pos < buf.size() && buf[pos] != '\n') out.push_back((char)buf[pos++]);
        if (pos < buf.size()) pos++;
        return true;
    };
    std::string ln;
    if (!line(ln) || (ln != "#?RADIANCE" && ln != "#?RGBE"))
        return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: not a Radiance RGBE file");
    bool fmt_ok = false;
    for (;;) {
        if (!line(ln)) return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: truncated header");
        if (ln.empty()) break;
        if (ln == "FORMAT=32-bit_rle_rgbe") fmt_ok = true;
    }
    if (!fmt_ok) return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: unsupported format");
    if (!line(ln)) return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: missing resolution");
    int H = 0, W = 0;
    char ys[3] = {0}, xs[3] = {0};
    if (std::sscanf(ln.c_str(), "%2s %d %2s %d", ys, &H, xs, &W) != 4 || std::strcmp(ys, "-Y") != 0 ||
        std::strcmp(xs, "+X") != 0 || W <= 0 || H <= 0 || (int64_t)W * H > (1LL << 30))
        return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: unsupported resolution line");
    std::vector<float> out(3 * (size_t)W * H);
    auto put = [&](size_t px, const unsigned char *c) {
        if (c[3] != 0) {
            float f1 = std::ldexp(1.0f, (int)c[3] - (128 + 8));
            out[3 * px] = c[0] * f1;
            out[3 * px + 1] = c[1] * f1;
            out[3 * px + 2] = c[2] * f1;
        } else {
            out[3 * px] = out[3 * px + 1] = out[3 * px + 2] = 0.f;
        }
    };
    auto fail_trunc = [&]() { return rt_internal_error(RT_ERR_INVALID, "rt_hdr_load: truncated pixel data"); };
    std::vector<unsigned char> sl(4 * (size_t)W);
    bool flat = false;
    for (int y = 0; y < H; y++) {
        if (!flat) {
            if (pos + 4 > buf.size()) return fail_trunc();
            const unsigned char *c = &buf[pos];
            bool rle = W >= 8 && W < 32768 && c[0] == 2 && c[1] == 2 && !(c[2] & 0x80) && ((c[2] << 8) | c[3]) == W;
            if (!rle) flat = true;   // the rest of the image is flat pixels
        }
        if (flat) {
            if (pos + 4 * (size_t)W > buf.size()) return fail_trunc();
            for (int x = 0; x < W; x++) put((size_t)y * W + x, &buf[pos + 4 * (size_t)x]);
            pos += 4 * (size_t)W;
            continue;
        }
        pos += 4;
        for (int k = 0; k < 4; k++) {
            int x = 0;
            while (x < W) {
                if (pos >= buf.size()) return fail_trunc();
                int count = buf[pos++];
                if (count > 128) {
                    count -= 128;
                    if (pos >= buf.size() || x + count > W) return fail_trunc();
                    unsigned char v = buf[pos++];
                    for (int i = 0; i < count; i++) sl[4 * (size_t)(x++) + k] = v;
                } else {
                    if (count == 0 || x + count > W || pos + count > buf.size()) return fail_trunc();
                    for (int i = 0; i < count; i++) sl[4 * (size_t)(x++) + k] = buf[pos++];
                }
            }
        }
        for (int x = 0; x < W; x++) put((size_t)y * W + x, &sl[4 * (size_t)x]);
    }
    float *p = (float *)std::malloc(out.size() * sizeof(float));
    if (!p) return rt_internal_error(RT_ERR_NOMEM, "rt_hdr_load: out of host memory");
    std::memcpy(p, out.data(), out.size() * sizeof(float));
    *rgb = p;
    *width = W;
    *height = H;
    return RT_OK;
}

extern "C" void rt_host_free(void *p) { std::free(p); }
