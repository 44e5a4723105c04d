// Mesh input: Wavefront OBJ files with MTL materials into host arrays
// (edxr_load_obj).  The reference loads meshes with Mesh::LoadMesh
// (Mesh.cpp:11-34) over EDXUtil's ObjMesh, which it does not include; the
// conventions below are this build's and are stated in include/edxr.h.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "edxr.h"
#include "edxr_internal.h"

namespace {

struct Material
{
    std::string name;
    float kd[3] = { 1.0f, 1.0f, 1.0f };
    std::string map;  // map_Kd image path, resolved against the MTL's folder
};

struct Image
{
    int w = 0, h = 0;
    std::vector<float> rgba;  // row 0 at v = 0 (the image's bottom row)
};

edxr_status obj_fail(edxr_status s, const std::string& msg)
{
    edxr::record_error(msg.c_str());
    return s;
}

std::string folder_of(const std::string& path)
{
    const size_t k = path.find_last_of("/\\");
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

std::string resolve(const std::string& folder, const std::string& p)
{
    if (p.empty() || p[0] == '/')
        return p;
    return folder + p;
}

// Binary PPM (P6), 8-bit channels; stored top row first.
bool load_ppm(const std::string& path, Image& img)
{
    std::ifstream in(path, std::ios::binary);
    if (!in)
        return false;
    std::string magic;
    in >> magic;
    if (magic != "P6")
        return false;
    auto next_int = [&](int& v) {
        for (;;)
        {
            in >> std::ws;
            if (in.peek() == '#')
            {
                std::string line;
                std::getline(in, line);
                continue;
            }
            in >> v;
            return (bool)in;
        }
    };
    int w, h, maxv;
    if (!next_int(w) || !next_int(h) || !next_int(maxv) || w <= 0 || h <= 0 || maxv <= 0 || maxv > 255)
        return false;
    in.get();  // the single whitespace before the samples
    std::vector<unsigned char> px((size_t)w * h * 3);
    in.read(reinterpret_cast<char*>(px.data()), (std::streamsize)px.size());
    if (!in)
        return false;
    img.w = w;
    img.h = h;
    img.rgba.resize((size_t)w * h * 4);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
        {
            const unsigned char* s = &px[((size_t)(h - 1 - y) * w + x) * 3];
            float* d = &img.rgba[((size_t)y * w + x) * 4];
            d[0] = s[0] / (float)maxv;
            d[1] = s[1] / (float)maxv;
            d[2] = s[2] / (float)maxv;
            d[3] = 1.0f;
        }
    return true;
}

uint32_t le32(const unsigned char* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
uint16_t le16(const unsigned char* p) { return (uint16_t)(p[0] | (p[1] << 8)); }

// Uncompressed BMP, 24 or 32 bits per pixel (BGR(A)); rows stored bottom
// first unless the height is negative.
bool load_bmp(const std::string& path, Image& img)
{
    std::ifstream in(path, std::ios::binary);
    if (!in)
        return false;
    std::vector<unsigned char> f((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (f.size() < 54 || f[0] != 'B' || f[1] != 'M')
        return false;
    const uint32_t off = le32(&f[10]);
    const int32_t w = (int32_t)le32(&f[18]), hraw = (int32_t)le32(&f[22]);
    const uint16_t bpp = le16(&f[28]);
    const uint32_t comp = le32(&f[30]);
    if (w <= 0 || hraw == 0 || (bpp != 24 && bpp != 32) || (comp != 0 && comp != 3))
        return false;
    const int h = hraw < 0 ? -hraw : hraw;
    const size_t row = ((size_t)w * (bpp / 8) + 3) & ~(size_t)3;
    if ((size_t)off + row * h > f.size())
        return false;
    img.w = w;
    img.h = h;
    img.rgba.resize((size_t)w * h * 4);
    for (int y = 0; y < h; y++)
    {
        const int fy = hraw > 0 ? y : h - 1 - y;  // file row holding image row y counted from the bottom
        const unsigned char* r = &f[off + row * fy];
        for (int x = 0; x < w; x++)
        {
            const unsigned char* s = r + (size_t)x * (bpp / 8);
            float* d = &img.rgba[((size_t)y * w + x) * 4];
            d[0] = s[2] / 255.0f;
            d[1] = s[1] / 255.0f;
            d[2] = s[0] / 255.0f;
            d[3] = bpp == 32 ? s[3] / 255.0f : 1.0f;
        }
    }
    return true;
}

bool load_image(const std::string& path, Image& img)
{
    const size_t n = path.size();
    auto ends = [&](const char* e) {
        const size_t m = std::strlen(e);
        if (n < m)
            return false;
        for (size_t i = 0; i < m; i++)
            if (std::tolower((unsigned char)path[n - m + i]) != e[i])
                return false;
        return true;
    };
    if (ends(".bmp"))
        return load_bmp(path, img);
    if (ends(".ppm"))
        return load_ppm(path, img);
    return false;
}

void load_mtl(const std::string& path, std::vector<Material>& mats)
{
    std::ifstream in(path);
    if (!in)
        return;
    const std::string folder = folder_of(path);
    std::string line;
    while (std::getline(in, line))
    {
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag))
            continue;
        if (tag == "newmtl")
        {
            Material m;
            ls >> m.name;
            mats.push_back(m);
        }
        else if (!mats.empty() && tag == "Kd")
            ls >> mats.back().kd[0] >> mats.back().kd[1] >> mats.back().kd[2];
        else if (!mats.empty() && tag == "map_Kd")
        {
            // options may precede the file name: keep the last token
            std::string tok, last;
            while (ls >> tok)
                last = tok;
            mats.back().map = resolve(folder, last);
        }
    }
}

struct Corner
{
    long long v, t, n;
};

// One "v/t/n" corner; indices are 1-based, negative ones count from the end.
bool parse_corner(const std::string& tok, size_t nv, size_t nt, size_t nn, Corner& c)
{
    long long idx[3] = { 0, 0, 0 };
    int part = 0;
    size_t i = 0;
    while (i <= tok.size() && part < 3)
    {
        const size_t j = tok.find('/', i);
        const std::string s = tok.substr(i, j == std::string::npos ? std::string::npos : j - i);
        if (!s.empty())
            idx[part] = std::strtoll(s.c_str(), nullptr, 10);
        part++;
        if (j == std::string::npos)
            break;
        i = j + 1;
    }
    auto fix = [](long long k, size_t count) -> long long {
        if (k > 0)
            return k - 1 < (long long)count ? k - 1 : -2;
        if (k < 0)
            return (long long)count + k >= 0 ? (long long)count + k : -2;
        return -1;  // absent
    };
    c.v = fix(idx[0], nv);
    c.t = fix(idx[1], nt);
    c.n = fix(idx[2], nn);
    return c.v >= 0 && c.t != -2 && c.n != -2;
}

struct CornerHash
{
    size_t operator()(const Corner& c) const
    {
        return std::hash<long long>()(c.v * 1000003LL ^ (c.t + 7) * 998244353LL ^ (c.n + 13));
    }
};
struct CornerEq
{
    bool operator()(const Corner& a, const Corner& b) const { return a.v == b.v && a.t == b.t && a.n == b.n; }
};

template <typename T>
T* copy_out(const std::vector<T>& v)
{
    T* p = static_cast<T*>(std::malloc(sizeof(T) * (v.empty() ? 1 : v.size())));
    if (p && !v.empty())
        std::memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
}

}  // namespace

extern "C" {

edxr_status edxr_load_obj(const char* path, const float pos[3], const float scale[3], const float rot_deg[3],
                          edxr_obj_mesh** out)
{
    if (!path || !out)
        return obj_fail(EDXR_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    std::ifstream in(path);
    if (!in)
        return obj_fail(EDXR_ERR_INVALID_ARG, std::string("cannot open ") + path);
    const std::string folder = folder_of(path);
    std::vector<float> P, T, N;  // as read
    std::vector<Material> mats;  // slot 0: the default white material
    mats.push_back(Material());
    std::unordered_map<std::string, uint32_t> by_name;
    uint32_t current = 0;
    std::vector<Corner> corners;  // per output vertex
    std::unordered_map<Corner, uint32_t, CornerHash, CornerEq> vmap;
    std::vector<uint32_t> idx, tex;
    std::string line;
    long long lineno = 0;
    while (std::getline(in, line))
    {
        lineno++;
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag) || tag[0] == '#')
            continue;
        if (tag == "v")
        {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            P.insert(P.end(), { x, y, z });
        }
        else if (tag == "vt")
        {
            float u = 0, v = 0;
            ls >> u >> v;
            T.insert(T.end(), { u, v });
        }
        else if (tag == "vn")
        {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            N.insert(N.end(), { x, y, z });
        }
        else if (tag == "mtllib")
        {
            std::string name;
            while (ls >> name)
            {
                const size_t first = mats.size();
                load_mtl(resolve(folder, name), mats);
                for (size_t m = first; m < mats.size(); m++)
                    by_name[mats[m].name] = (uint32_t)m;
            }
        }
        else if (tag == "usemtl")
        {
            std::string name;
            ls >> name;
            auto it = by_name.find(name);
            current = it == by_name.end() ? 0u : it->second;
        }
        else if (tag == "f")
        {
            std::vector<uint32_t> face;
            std::string tok;
            while (ls >> tok)
            {
                Corner c;
                if (!parse_corner(tok, P.size() / 3, T.size() / 2, N.size() / 3, c))
                    return obj_fail(EDXR_ERR_INVALID_ARG,
                                    std::string(path) + ": bad face corner at line " + std::to_string(lineno));
                auto it = vmap.find(c);
                if (it == vmap.end())
                {
                    it = vmap.emplace(c, (uint32_t)corners.size()).first;
                    corners.push_back(c);
                }
                face.push_back(it->second);
            }
            // fan triangulation
            for (size_t k = 2; k < face.size(); k++)
            {
                idx.insert(idx.end(), { face[0], face[k - 1], face[k] });
                tex.push_back(current);
            }
        }
    }
    if (corners.size() >= (1ull << 31) || tex.size() >= (1ull << 28))
        return obj_fail(EDXR_ERR_INVALID_ARG, "mesh too large");

    // scale, rotate about x, y, z (degrees), translate
    const float s[3] = { scale ? scale[0] : 1.0f, scale ? scale[1] : 1.0f, scale ? scale[2] : 1.0f };
    const double rad = 3.14159265358979323846 / 180.0;
    const double ax = rot_deg ? rot_deg[0] * rad : 0.0, ay = rot_deg ? rot_deg[1] * rad : 0.0,
                 az = rot_deg ? rot_deg[2] * rad : 0.0;
    auto rotate = [&](double v[3]) {
        double y = v[1] * std::cos(ax) - v[2] * std::sin(ax), z = v[1] * std::sin(ax) + v[2] * std::cos(ax);
        v[1] = y; v[2] = z;
        double x = v[0] * std::cos(ay) + v[2] * std::sin(ay);
        z = -v[0] * std::sin(ay) + v[2] * std::cos(ay);
        v[0] = x; v[2] = z;
        x = v[0] * std::cos(az) - v[1] * std::sin(az);
        y = v[0] * std::sin(az) + v[1] * std::cos(az);
        v[0] = x; v[1] = y;
    };
    const size_t nv = corners.size();
    std::vector<float> op(3 * nv), on(3 * nv, 0.0f), ouv(2 * nv, 0.0f);
    std::vector<double> acc(3 * nv, 0.0);  // face normals of corners without one
    for (size_t i = 0; i < nv; i++)
    {
        const Corner& c = corners[i];
        double p[3] = { P[3 * c.v] * (double)s[0], P[3 * c.v + 1] * (double)s[1], P[3 * c.v + 2] * (double)s[2] };
        rotate(p);
        for (int q = 0; q < 3; q++)
            op[3 * i + q] = (float)(p[q] + (pos ? pos[q] : 0.0f));
        if (c.t >= 0)
        {
            ouv[2 * i] = T[2 * c.t];
            ouv[2 * i + 1] = T[2 * c.t + 1];
        }
    }
    for (size_t t = 0; t < idx.size() / 3; t++)
    {
        const float* a = &op[3 * idx[3 * t]];
        const float* b = &op[3 * idx[3 * t + 1]];
        const float* c = &op[3 * idx[3 * t + 2]];
        const double e1[3] = { (double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2] };
        const double e2[3] = { (double)c[0] - a[0], (double)c[1] - a[1], (double)c[2] - a[2] };
        const double n[3] = { e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                              e1[0] * e2[1] - e1[1] * e2[0] };
        for (int k = 0; k < 3; k++)
            for (int q = 0; q < 3; q++)
                acc[3 * idx[3 * t + k] + q] += n[q];
    }
    for (size_t i = 0; i < nv; i++)
    {
        const Corner& c = corners[i];
        double n[3];
        if (c.n >= 0)
        {
            // normals transform with the inverse transpose of the scale
            n[0] = N[3 * c.n] / (double)s[0];
            n[1] = N[3 * c.n + 1] / (double)s[1];
            n[2] = N[3 * c.n + 2] / (double)s[2];
            rotate(n);
        }
        else
        {
            n[0] = acc[3 * i];
            n[1] = acc[3 * i + 1];
            n[2] = acc[3 * i + 2];
        }
        const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int q = 0; q < 3; q++)
            on[3 * i + q] = len > 0.0 ? (float)(n[q] / len) : 0.0f;
    }

    edxr_obj_mesh* m = static_cast<edxr_obj_mesh*>(std::calloc(1, sizeof(edxr_obj_mesh)));
    if (!m)
        return obj_fail(EDXR_ERR_OUT_OF_MEMORY, "out of host memory");
    m->num_vertices = (uint32_t)nv;
    m->num_triangles = (uint32_t)tex.size();
    m->num_textures = (uint32_t)mats.size();
    m->positions = copy_out(op);
    m->normals = copy_out(on);
    m->uvs = copy_out(ouv);
    m->indices = copy_out(idx);
    m->texture_ids = copy_out(tex);
    m->textures = static_cast<edxr_texture*>(std::calloc(mats.size(), sizeof(edxr_texture)));
    bool ok = m->positions && m->normals && m->uvs && m->indices && m->texture_ids && m->textures;
    for (size_t k = 0; ok && k < mats.size(); k++)
    {
        Image img;
        if (mats[k].map.empty() || !load_image(mats[k].map, img))
        {
            img.w = img.h = 1;
            img.rgba = { mats[k].kd[0], mats[k].kd[1], mats[k].kd[2], 1.0f };
        }
        edxr_texture& t = m->textures[k];
        t.width = (uint32_t)img.w;
        t.height = (uint32_t)img.h;
        t.format = EDXR_TEXTURE_RGBA32F;
        t.texels = copy_out(img.rgba);
        ok = t.texels != nullptr;
    }
    if (!ok)
    {
        edxr_free_obj(m);
        return obj_fail(EDXR_ERR_OUT_OF_MEMORY, "out of host memory");
    }
    *out = m;
    return EDXR_OK;
}

void edxr_free_obj(edxr_obj_mesh* m)
{
    if (!m)
        return;
    std::free(m->positions);
    std::free(m->normals);
    std::free(m->uvs);
    std::free(m->indices);
    std::free(m->texture_ids);
    if (m->textures)
        for (uint32_t k = 0; k < m->num_textures; k++)
            std::free(const_cast<void*>(m->textures[k].texels));
    std::free(m->textures);
    std::free(m);
}

}  // extern "C"
