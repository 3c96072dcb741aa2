// Scene files in the reference's formats (declared in loader.h).
#include "loader.h"

#include <charconv>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <sys/stat.h>
#include <unistd.h>

#include "image_io.h"

namespace cpppt_gb300 {
namespace hostimpl {
namespace {

// ---------------------------------------------------------------------------
// Reference file formats (Loader, src/loader/loader.h:20-374)
// ---------------------------------------------------------------------------
std::string trim(const std::string& s) {
    size_t i = s.find_first_not_of(" \n\t\r");
    if (i == std::string::npos) return "";
    size_t j = s.find_last_not_of(" \n\t\r");
    return s.substr(i, j - i + 1);
}

// texture string -> rgb (ConstantTexture); bw: keep the first channel only
void parse_tex(const std::string& tex, bool bw, bool srgb, float out[3]) {
    if (tex.rfind("rgb", 0) == 0) {  // loader.h:47-61: rgb(...) is never sRGB-converted
        size_t c1 = tex.find(',');
        size_t c2 = tex.find(',', c1 + 1);
        if (tex.size() < 5 || c1 == std::string::npos || c2 == std::string::npos)
            throw Fail(PT_ERR_IO, "bad texture: " + tex);
        out[0] = (float)std::atof(tex.substr(4, c1 - 4).c_str());
        out[1] = (float)std::atof(tex.substr(c1 + 1, c2 - c1 - 1).c_str());
        out[2] = (float)std::atof(tex.substr(c2 + 1, tex.size() - c2 - 2).c_str());
        if (bw) out[1] = out[2] = out[0];
        return;
    }
    if (tex.rfind("float", 0) == 0) {  // loader.h:62-77
        if (tex.size() < 7) throw Fail(PT_ERR_IO, "bad texture: " + tex);
        float r = (float)std::atof(tex.substr(6, tex.size() - 7).c_str());
        if (srgb) r = srgb_to_linear_ref(r);  // pixel_ops::srgb2linear, rgb_image.h:122-128
        out[0] = out[1] = out[2] = r;
        return;
    }
    throw Fail(PT_ERR_IO, "Unknown type of tex: " + tex);
}

// An image(...) texture: the file decoded (image_io.cpp) into the pixels
// Image<Vec3> (rgb) or Image<float> holds (loader.h:78-92: the colour space
// is sRGB for albedo and emission, linear for roughness, metal and normal
// maps); identical requests share one texture.  Returns its id.
int load_image_texture(LoadedScene& L, const std::string& dir, const std::string& tex, bool rgb, bool srgb) {
    if (tex.size() < 8 || tex.back() != ')') throw Fail(PT_ERR_IO, "bad texture: " + tex);
    const std::string path = dir + tex.substr(6, tex.size() - 7);
    const std::string key = path + (rgb ? "|rgb" : "|bw") + (srgb ? "|srgb" : "|lin");
    auto it = L.tex_cache.find(key);
    if (it != L.tex_cache.end()) return it->second;
    if (L.tx.info.size() >= kNoTex) throw Fail(PT_ERR_LIMIT, "more than 254 image textures");
    DecodedImage im;
    try {
        im = decode_image_file(path);
    } catch (std::runtime_error& e) {
        throw Fail(PT_ERR_IO, e.what());
    }
    std::vector<float> px;
    texture_pixels(im, rgb, srgb, px);
    const int id = (int)L.tx.info.size();
    L.tx.info.push_back(make_int4((int)L.tx.px.size(), im.w, im.h, rgb ? 3 : 1));
    L.tx.px.insert(L.tx.px.end(), px.begin(), px.end());
    L.tex_cache[key] = id;
    return id;
}

std::string dir_of(const std::string& f) {
    size_t i = f.find_last_of("/\\");
    return i == std::string::npos ? std::string("./") : f.substr(0, i) + "/";
}

// .ptobj meshes (loader.h:209-251): "nv nf TRIANGLE_MESH", nv lines of
// position (3), uv (2), normal (3), tangent (3), nf lines of three vertex
// indices.  The file is read in one piece and parsed with std::from_chars,
// which rounds like the reference's istream >> float (both correctly
// rounded), about ten times faster than line-by-line stream extraction.
// Parsed meshes are cached next to the source as <file>.gbbin (positions,
// normals, tangents, faces), keyed by the source's size and modification
// time; a stale or unreadable cache is ignored and rewritten.
struct MeshArrays {
    std::vector<float> v, n, t;  // 3 per vertex
    std::vector<float> uv;       // 2 per vertex
    std::vector<int32_t> f;      // 3 per face
};

const char kMeshCacheMagic[8] = {'G', 'B', 'P', 'T', 'O', 'B', 'J', '2'};
bool g_mesh_cache = true;

struct FileStamp {
    long long size = -1, mtime_ns = 0;
};
FileStamp file_stamp(const std::string& path) {
    struct stat st;
    FileStamp fs;
    if (stat(path.c_str(), &st) != 0) return fs;
    fs.size = (long long)st.st_size;
    fs.mtime_ns = (long long)st.st_mtim.tv_sec * 1000000000LL + (long long)st.st_mtim.tv_nsec;
    return fs;
}

bool read_mesh_cache(const std::string& cpath, const FileStamp& src, MeshArrays& M) {
    std::ifstream f(cpath, std::ios::binary);
    if (!f) return false;
    char magic[8];
    long long size = 0, mtime = 0;
    int32_t nv = 0, nf = 0;
    f.read(magic, 8);
    f.read(reinterpret_cast<char*>(&size), sizeof(size));
    f.read(reinterpret_cast<char*>(&mtime), sizeof(mtime));
    f.read(reinterpret_cast<char*>(&nv), sizeof(nv));
    f.read(reinterpret_cast<char*>(&nf), sizeof(nf));
    if (!f || std::memcmp(magic, kMeshCacheMagic, 8) != 0 || size != src.size || mtime != src.mtime_ns || nv < 0 ||
        nf < 0)
        return false;
    M.v.resize(3 * (size_t)nv);
    M.n.resize(3 * (size_t)nv);
    M.t.resize(3 * (size_t)nv);
    M.uv.resize(2 * (size_t)nv);
    M.f.resize(3 * (size_t)nf);
    f.read(reinterpret_cast<char*>(M.v.data()), sizeof(float) * M.v.size());
    f.read(reinterpret_cast<char*>(M.n.data()), sizeof(float) * M.n.size());
    f.read(reinterpret_cast<char*>(M.t.data()), sizeof(float) * M.t.size());
    f.read(reinterpret_cast<char*>(M.uv.data()), sizeof(float) * M.uv.size());
    f.read(reinterpret_cast<char*>(M.f.data()), sizeof(int32_t) * M.f.size());
    return (bool)f;
}

void write_mesh_cache(const std::string& cpath, const FileStamp& src, const MeshArrays& M) {
    const std::string tmp = cpath + ".tmp" + std::to_string((long long)getpid());
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f) return;  // read-only directory: no cache
        const int32_t nv = (int32_t)(M.v.size() / 3), nf = (int32_t)(M.f.size() / 3);
        f.write(kMeshCacheMagic, 8);
        f.write(reinterpret_cast<const char*>(&src.size), sizeof(src.size));
        f.write(reinterpret_cast<const char*>(&src.mtime_ns), sizeof(src.mtime_ns));
        f.write(reinterpret_cast<const char*>(&nv), sizeof(nv));
        f.write(reinterpret_cast<const char*>(&nf), sizeof(nf));
        f.write(reinterpret_cast<const char*>(M.v.data()), sizeof(float) * M.v.size());
        f.write(reinterpret_cast<const char*>(M.n.data()), sizeof(float) * M.n.size());
        f.write(reinterpret_cast<const char*>(M.t.data()), sizeof(float) * M.t.size());
        f.write(reinterpret_cast<const char*>(M.uv.data()), sizeof(float) * M.uv.size());
        f.write(reinterpret_cast<const char*>(M.f.data()), sizeof(int32_t) * M.f.size());
        if (!f) {
            f.close();
            std::remove(tmp.c_str());
            return;
        }
    }
    if (std::rename(tmp.c_str(), cpath.c_str()) != 0) std::remove(tmp.c_str());
}

// Next whitespace-separated token of [p, end) on the current line.
struct LineCursor {
    const char* p;
    const char* end;  // end of line
    bool next(const char*& tb, const char*& te) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
        if (p >= end) return false;
        tb = p;
        while (p < end && *p != ' ' && *p != '\t' && *p != '\r') p++;
        te = p;
        return true;
    }
};

void parse_ptobj_text(const std::string& path, MeshArrays& M) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Fail(PT_ERR_IO, "cannot open " + path);
    std::string buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    const char* p = buf.data();
    const char* const end = p + buf.size();
    auto next_line = [&](const char* what) {
        if (p >= end) throw Fail(PT_ERR_IO, std::string("Insuficient number of lines when reading ") + what);
        const char* e = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        if (!e) e = end;
        LineCursor c{p, e};
        p = e < end ? e + 1 : end;
        return c;
    };
    LineCursor h = next_line("file");
    const char *tb, *te;
    int nv = 0, nf = 0;
    if (h.next(tb, te)) std::from_chars(tb, te, nv);
    if (h.next(tb, te)) std::from_chars(tb, te, nf);
    if (!h.next(tb, te) || std::string(tb, te) != "TRIANGLE_MESH")
        throw Fail(PT_ERR_IO, "Unknown mesh type in " + path);
    if (nv < 0 || nf < 0) throw Fail(PT_ERR_IO, "negative counts in " + path);
    M.v.resize(3 * (size_t)nv);
    M.n.resize(3 * (size_t)nv);
    M.t.resize(3 * (size_t)nv);
    M.uv.resize(2 * (size_t)nv);
    M.f.resize(3 * (size_t)nf);
    for (int i = 0; i < nv; i++) {
        LineCursor c = next_line("verts");
        float x[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 11 && c.next(tb, te); k++) std::from_chars(tb, te, x[k]);
        std::memcpy(&M.v[3 * (size_t)i], x, 12);
        std::memcpy(&M.uv[2 * (size_t)i], x + 3, 8);
        std::memcpy(&M.n[3 * (size_t)i], x + 5, 12);
        std::memcpy(&M.t[3 * (size_t)i], x + 8, 12);
    }
    for (int i = 0; i < nf; i++) {
        LineCursor c = next_line("faces");
        int ix[3] = {-1, -1, -1};
        for (int k = 0; k < 3 && c.next(tb, te); k++) std::from_chars(tb, te, ix[k]);
        for (int k = 0; k < 3; k++)
            if (ix[k] < 0 || ix[k] >= nv) throw Fail(PT_ERR_IO, "face index out of range in " + path);
        std::memcpy(&M.f[3 * (size_t)i], ix, 12);
    }
}

void parse_ptobj(const std::string& path, LoadedScene& L, int mat) {
    MeshArrays M;
    const FileStamp src = file_stamp(path);
    const std::string cpath = path + ".gbbin";
    if (!(g_mesh_cache && src.size >= 0 && read_mesh_cache(cpath, src, M))) {
        parse_ptobj_text(path, M);
        if (g_mesh_cache && src.size >= 0) write_mesh_cache(cpath, src, M);
    }
    const int base = (int)(L.v.size() / 3);
    L.v.insert(L.v.end(), M.v.begin(), M.v.end());
    L.n.insert(L.n.end(), M.n.begin(), M.n.end());
    L.t.insert(L.t.end(), M.t.begin(), M.t.end());
    L.tx.uv.insert(L.tx.uv.end(), M.uv.begin(), M.uv.end());
    for (int32_t ix : M.f) L.tri.push_back(base + ix);
    L.tri_mat.insert(L.tri_mat.end(), M.f.size() / 3, mat);
}

int parse_ptmat(const std::string& path, LoadedScene& L, std::unordered_map<std::string, int>& cache) {
    auto it = cache.find(path);  // loader.h:147-150: materials are shared by file name
    if (it != cache.end()) return it->second;
    std::ifstream f(path);
    if (!f) throw Fail(PT_ERR_IO, "cannot open " + path);
    std::string word;
    f >> word;
    pt_material m{};
    const std::string dir = dir_of(path);
    uint32_t tex = kNoTextures;  // DevMaterial::tex
    float emit_intensity = 0.f;
    // an image(...) texture goes to the slot `shift`; returns whether it was one
    auto image = [&](const std::string& t, bool rgb, bool srgb, int shift) {
        if (t.rfind("image", 0) != 0) return false;
        const uint32_t id = (uint32_t)load_image_texture(L, dir, t, rgb, srgb);
        tex = (tex & ~(0xffu << shift)) | (id << shift);
        return true;
    };
    if (word == "DISNEY") {  // loader.h:154-180
        std::string albedo, spec, rough, metal, transp, ior, normal, alpha;
        f >> albedo >> spec >> rough >> metal >> transp >> ior >> normal >> alpha;
        float a[3] = {0.f, 0.f, 0.f}, r[3] = {0.f, 0.f, 0.f}, me[3] = {0.f, 0.f, 0.f}, io[3] = {0.f, 0.f, 0.f};
        if (!image(albedo, true, true, 0)) parse_tex(albedo, false, true, a);
        if (!image(rough, false, false, 8)) parse_tex(rough, true, false, r);
        if (!image(metal, false, false, 16)) parse_tex(metal, true, false, me);
        image(normal, true, false, 24);  // a constant normal map is the identity here
        if (ior.rfind("image", 0) != 0) parse_tex(ior, true, true, io);  // unused by the BxDFs
        // standard_material.h:46-61: Diffuse when metal < 0.1, else Glossy(roughness)
        m.kind = (double)me[0] < 0.1 ? PT_MAT_DIFFUSE : PT_MAT_GGX;
        std::memcpy(m.rgb, a, 12);
        m.roughness = r[0];
        m.ior = io[0];
    } else if (word == "EMISSION") {  // loader.h:181-201
        std::string col, inten;
        f >> col >> inten;
        float c[3] = {0.f, 0.f, 0.f};
        const bool textured = image(col, true, true, 0);
        if (!textured) parse_tex(col, false, true, c);
        m.kind = PT_MAT_EMISSIVE;
        std::memcpy(m.rgb, c, 12);
        m.intensity = (float)std::atof(inten.substr(6, inten.size() - 7).c_str());
        emit_intensity = m.intensity;
        if (textured) m.rgb[0] = m.rgb[1] = m.rgb[2] = 1.0f;  // a lit placeholder; the texture decides
    } else if (word == "DIELECTRIC") {  // extension: RefractionBxDF(ior)
        std::string ior;
        f >> ior;
        float io[3];
        parse_tex(ior, true, false, io);
        m.kind = PT_MAT_DIELECTRIC;
        m.ior = io[0];
        m.rgb[0] = m.rgb[1] = m.rgb[2] = 1.0f;
    } else {
        throw Fail(PT_ERR_IO, "Wrong bsdf type: " + word);
    }
    L.mats.push_back(m);
    L.tx.mat_tex.push_back(tex);
    L.tx.emit_intensity.push_back(emit_intensity);
    int id = (int)L.mats.size() - 1;
    cache[path] = id;
    return id;
}

}  // namespace

void load_files(const std::string& settings_file, LoadedScene& L, pt_render_desc* rs, std::string& output) {
    std::ifstream f(settings_file);
    if (!f) throw Fail(PT_ERR_IO, "cannot open " + settings_file);
    std::string line, scene_name;
    int spp = 1, rx = 256, ry = 256;  // RenderSettings defaults (renderer.h:19-22)
    while (std::getline(f, line)) {  // loader.h:256-311
        line = line.substr(0, line.find('#'));
        std::istringstream s(line);
        std::string type;
        s >> type;
        if (type == "renderer") {
            std::string r;
            s >> r;
            if (r != "pathtracer_mis" && r != "pathtracer" && r != "pure_pt" && r != "ppg" && r != "debug" &&
                r != "lighttracer" && r != "pathtracer_mlt" && r != "lighttracer_mlt" && r != "photonmapping" &&
                r != "validation")
                throw Fail(PT_ERR_IO, "Unknown renderer type: " + r);
        } else if (type == "spp") {
            s >> spp;
        } else if (type == "resolution") {
            s >> rx >> ry;
        } else if (type == "scene") {
            s >> scene_name;
        } else if (type == "output") {
            s >> output;
        } else if (!type.empty()) {
            throw Fail(PT_ERR_IO, "Unknown render setting: " + type);
        }
    }
    std::ifstream sf(scene_name);
    if (!sf) throw Fail(PT_ERR_IO, "cannot open scene " + scene_name);
    const std::string dir = dir_of(scene_name);
    std::unordered_map<std::string, int> cache;
    while (std::getline(sf, line)) {  // loader.h:330-351
        line = trim(line.substr(0, line.find('#')));
        std::istringstream s(line);
        std::string type;
        s >> type;
        if (type == "camera") {
            pt_camera& c = L.cam;
            s >> c.origin[0] >> c.origin[1] >> c.origin[2] >> c.at[0] >> c.at[1] >> c.at[2] >> c.up[0] >> c.up[1] >>
                c.up[2] >> c.tan_fovy;
            L.has_camera = true;
        } else if (type == "obj") {
            std::string obj, mat;
            s >> obj >> mat;
            const size_t first = L.tri_mat.size();
            parse_ptobj(dir + obj, L, 0);
            int m = parse_ptmat(dir + mat, L, cache);
            for (size_t i = first; i < L.tri_mat.size(); i++) L.tri_mat[i] = m;
        } else if (type == "light") {
            throw Fail(PT_ERR_IO, "point lights are not supported");
        } else if (!type.empty()) {
            throw Fail(PT_ERR_IO, "Unknown scene obj: " + type);
        }
    }
    if (!L.has_camera) throw Fail(PT_ERR_IO, "scene has no camera");
    L.cam.width = rx;
    L.cam.height = ry;
    rs->spp = spp * spp;  // pathtracerMIS.h:148-149: spp x spp samples per pixel
    rs->max_depth = 32;
    rs->rr_start = 3;
    rs->seed = 0;
    rs->mode = PT_MODE_MIS;
    rs->flags = 0;
}

void set_mesh_cache(bool enabled) { g_mesh_cache = enabled; }

}  // namespace hostimpl
}  // namespace cpppt_gb300
