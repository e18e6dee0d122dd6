// scene_file.cpp -- readers for the reference's scene (*.scene) and camera
// (*.scr) files.
//
// The reference ships these files (example/*.scene, example/*.scr; the camera
// grammar in doc/ebnf-camera.txt) but its read_scene / read_camera ignore the
// path and return built-in values (src/scene.rs:20, src/camera.rs:108).  This
// reader turns the files into the C ABI's structs, as the reference's types
// would hold them:
//   material (type solid): Material {emittance, transmittance, ior} +
//       Surface::new_simple(reflectance, specularrefl, diffuseness, metalness,
//       roughness = smoothness) -- the built-in version of ex-11.1 passes 0.0
//       where the file says smoothness 0.0 (e.g. its silver mirror);
//   light point / parallelogram / sun: Color::normalize(color), flux (or
//       power), position; parallelogram and sun add dir1, dir2 and
//       nvec = normalize(dir1 x dir2); sun adds dir = normalize(ldir);
//   object plain: nvec = normalize(normal), dist = -(nvec . position);
//       sphere: center, radius; polygon / parallelogram: pos1..3 (vertex
//       names from the vertex section, or literal vectors), built as
//       Shape::new_polygon / new_parallelogram (geometry.rs:93-115).
// The syntax is the indentation-based subset these files use: top-level
// "section:" lines, "- key: value" list items with further "key: value"
// lines, values that are numbers, [x, y, z] vectors, names or yes/no, and
// '#' comments.  Sections the reference's model has no place for (air,
// ambient_light) are read and ignored.
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/ppm_api.h"

namespace {

thread_local std::string g_parse_error;

struct Entry {
    std::map<std::string, std::string> kv;
    int line = 0;
};

struct Doc {
    std::map<std::string, std::vector<Entry>> lists;   // "- item" sections
    std::map<std::string, Entry> maps;                // plain key/value sections
    Entry top;                                        // top-level key: value
};

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

std::string norm_key(std::string k) {
    std::string o;
    for (char c : k)
        if (c != '_') o += (char)std::tolower((unsigned char)c);
    return o;
}

bool fail(int line, const std::string &msg) {
    g_parse_error = "line " + std::to_string(line) + ": " + msg;
    return false;
}

int err(int line, const std::string &msg) {
    fail(line, msg);
    return PPM_ERR_INVALID_ARG;
}

bool parse_doc(const char *text, Doc &d) {
    std::string cur_section;
    Entry *cur = nullptr;
    int ln = 0;
    const char *p = text;
    while (*p) {
        const char *e = std::strchr(p, '\n');
        std::string line = e ? std::string(p, e - p) : std::string(p);
        p = e ? e + 1 : p + line.size();
        ln++;
        size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        if (trim(line).empty()) continue;
        const bool indented = std::isspace((unsigned char)line[0]);
        std::string body = trim(line);
        bool item = false;
        if (body[0] == '-') {
            item = true;
            body = trim(body.substr(1));
        }
        size_t colon = body.find(':');
        if (colon == std::string::npos) return fail(ln, "expected 'key: value'");
        std::string key = norm_key(trim(body.substr(0, colon)));
        std::string val = trim(body.substr(colon + 1));
        if (!indented && !item) {
            if (val.empty()) {        // section header
                cur_section = key;
                cur = nullptr;
            } else {
                d.top.kv[key] = val;
                cur_section.clear();
                cur = nullptr;
            }
            continue;
        }
        if (cur_section.empty()) return fail(ln, "indented line outside a section");
        if (item) {
            d.lists[cur_section].push_back(Entry{});
            cur = &d.lists[cur_section].back();
            cur->line = ln;
        } else if (!cur) {
            cur = &d.maps[cur_section];
            cur->line = ln;
        }
        cur->kv[key] = val;
    }
    return true;
}

bool to_num(const std::string &s, double &v) {
    if (s.empty()) return false;
    char *end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

bool to_vec(const std::string &s, double v[3]) {
    std::string t = trim(s);
    if (t.size() < 2 || t.front() != '[' || t.back() != ']') return false;
    t = t.substr(1, t.size() - 2);
    int k = 0;
    size_t a = 0;
    while (k < 3) {
        size_t b = t.find(',', a);
        std::string f = trim(t.substr(a, b == std::string::npos ? std::string::npos : b - a));
        if (!to_num(f, v[k])) return false;
        k++;
        if (b == std::string::npos) break;
        a = b + 1;
    }
    return k == 3 && t.find(',', a) == std::string::npos;
}

bool get_num(const Entry &e, const char *key, double &v, bool required = true, double dflt = 0.0) {
    auto it = e.kv.find(key);
    if (it == e.kv.end()) {
        v = dflt;
        return required ? fail(e.line, std::string("missing '") + key + "'") : true;
    }
    if (!to_num(it->second, v)) return fail(e.line, std::string("'") + key + "' is not a number");
    return true;
}

bool get_vec(const Entry &e, const char *key, double v[3], const std::map<std::string, std::array<double, 3>> *names,
             bool required = true) {
    auto it = e.kv.find(key);
    if (it == e.kv.end()) {
        v[0] = v[1] = v[2] = 0.0;
        return required ? fail(e.line, std::string("missing '") + key + "'") : true;
    }
    if (to_vec(it->second, v)) return true;
    if (names) {
        auto n = names->find(it->second);
        if (n != names->end()) {
            for (int a = 0; a < 3; a++) v[a] = n->second[a];
            return true;
        }
    }
    return fail(e.line, std::string("'") + key + "' is not a vector" + (names ? " or a vertex name" : ""));
}

void normalize3(const double a[3], double o[3]) {   // Vector3::normalize: a * (1 / |a|)
    double n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    double r = n == 0.0 ? 0.0 : 1.0 / n;
    for (int k = 0; k < 3; k++) o[k] = a[k] * r;
}

void cross3(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}

void color_normalize(const double c[3], double o[3]) {   // Color::normalize (physics.rs:61-71)
    double r = c[0] >= 0.0 ? c[0] : 0.0, g = c[1] >= 0.0 ? c[1] : 0.0, b = c[2] >= 0.0 ? c[2] : 0.0;
    double m = r + g + b;
    if (m == 0.0) { o[0] = o[1] = o[2] = 1.0 / 3.0; return; }
    o[0] = r / m; o[1] = g / m; o[2] = b / m;
}

std::string get_str(const Entry &e, const char *key) {
    auto it = e.kv.find(key);
    return it == e.kv.end() ? std::string() : it->second;
}

}  // namespace

extern "C" const char *ppm_parse_error(void) { return g_parse_error.c_str(); }

extern "C" int ppm_scene_parse(const char *text, ppm_object *objs, int32_t *n_objs, ppm_material *mats,
                               int32_t *n_mats, ppm_light *lights, int32_t *n_lights) {
    g_parse_error.clear();
    if (!text || !n_objs || !n_mats || !n_lights) {
        g_parse_error = "null argument";
        return PPM_ERR_INVALID_ARG;
    }
    Doc d;
    if (!parse_doc(text, d)) return PPM_ERR_INVALID_ARG;
    std::vector<ppm_material> M;
    std::map<std::string, int> mat_index;
    for (const Entry &e : d.lists["material"]) {
        std::string type = get_str(e, "type"), name = get_str(e, "name");
        if (type != "solid") return err(e.line, "material type '" + type + "' (only solid)");
        ppm_material m;
        std::memset(&m, 0, sizeof m);
        double rough = 0.0;
        if (!get_vec(e, "emittance", m.emittance, nullptr, false) || !get_vec(e, "reflectance", m.color_diff, nullptr) ||
            !get_vec(e, "transmittance", m.transmittance, nullptr, false) ||
            !get_vec(e, "specularrefl", m.color_spec, nullptr, false) || !get_vec(e, "ior", m.ior, nullptr, false) ||
            !get_num(e, "diffuseness", m.scatter) || !get_num(e, "metalness", m.metalness, false) ||
            !get_num(e, "smoothness", rough, false))
            return PPM_ERR_INVALID_ARG;
        m.surface = PPM_SURF_SIMPLE;
        m.roughness = rough;
        ppm_material_derive(&m);
        if (name.empty()) return err(e.line, "material without a name");
        mat_index[name] = (int)M.size();
        M.push_back(m);
    }
    std::map<std::string, std::array<double, 3>> verts;
    std::vector<Entry> vsec = d.lists["vertex"];
    if (d.maps.count("vertex")) vsec.push_back(d.maps["vertex"]);   // "name: [x, y, z]" without '-'
    for (const Entry &e : vsec)
        for (const auto &kv : e.kv) {
            std::array<double, 3> v;
            if (!to_vec(kv.second, v.data())) return err(e.line, "vertex '" + kv.first + "' is not a vector");
            verts[kv.first] = v;
        }
    std::vector<ppm_light> L;
    for (const Entry &e : d.lists["light"]) {
        std::string type = get_str(e, "type");
        ppm_light l;
        std::memset(&l, 0, sizeof l);
        double col[3];
        if (!get_vec(e, "color", col, nullptr)) return PPM_ERR_INVALID_ARG;
        color_normalize(col, l.color);
        if (e.kv.count("flux")) { if (!get_num(e, "flux", l.flux)) return PPM_ERR_INVALID_ARG; }
        else if (!get_num(e, "power", l.flux)) return PPM_ERR_INVALID_ARG;
        if (!get_vec(e, "position", l.pos, &verts)) return PPM_ERR_INVALID_ARG;
        if (type == "point") {
            l.kind = PPM_LIGHT_POINT;
        } else if (type == "parallelogram" || type == "sun") {
            l.kind = type == "sun" ? PPM_LIGHT_SUN : PPM_LIGHT_PARALLELOGRAM;
            if (!get_vec(e, "dir1", l.dir1, nullptr) || !get_vec(e, "dir2", l.dir2, nullptr)) return PPM_ERR_INVALID_ARG;
            double c[3];
            cross3(l.dir1, l.dir2, c);
            normalize3(c, l.nvec);
            if (type == "sun") {
                double ld[3];
                if (!get_vec(e, "ldir", ld, nullptr)) return PPM_ERR_INVALID_ARG;
                normalize3(ld, l.dir);
            }
        } else {
            return err(e.line, "light type '" + type + "'");
        }
        L.push_back(l);
    }
    std::vector<ppm_object> O;
    for (const Entry &e : d.lists["object"]) {
        std::string type = get_str(e, "type"), mname = get_str(e, "material");
        auto mi = mat_index.find(mname);
        if (mi == mat_index.end()) return err(e.line, "unknown material '" + mname + "'");
        ppm_object o;
        std::memset(&o, 0, sizeof o);
        o.material = mi->second;
        if (type == "plain") {
            double n[3], p[3];
            if (!get_vec(e, "normal", n, nullptr) || !get_vec(e, "position", p, &verts)) return PPM_ERR_INVALID_ARG;
            o.shape = PPM_SHAPE_PLAIN;
            normalize3(n, o.nvec);
            o.dist = -(o.nvec[0] * p[0] + o.nvec[1] * p[1] + o.nvec[2] * p[2]);
        } else if (type == "sphere") {
            o.shape = PPM_SHAPE_SPHERE;
            if (!get_vec(e, "center", o.position, &verts) || !get_num(e, "radius", o.radius)) return PPM_ERR_INVALID_ARG;
        } else if (type == "polygon" || type == "parallelogram") {
            double p0[3], p1[3], p2[3];
            if (!get_vec(e, "pos1", p0, &verts) || !get_vec(e, "pos2", p1, &verts) || !get_vec(e, "pos3", p2, &verts))
                return PPM_ERR_INVALID_ARG;
            o.shape = type == "polygon" ? PPM_SHAPE_POLYGON : PPM_SHAPE_PARALLELOGRAM;
            for (int a = 0; a < 3; a++) {
                o.position[a] = p0[a];
                o.dir1[a] = p1[a] - p0[a];
                o.dir2[a] = p2[a] - p0[a];
            }
            double c[3];
            cross3(o.dir1, o.dir2, c);
            normalize3(c, o.nvec);
        } else {
            return err(e.line, "object type '" + type + "'");
        }
        O.push_back(o);
    }
    const bool fill = objs || mats || lights;
    if (fill && (*n_objs < (int32_t)O.size() || *n_mats < (int32_t)M.size() || *n_lights < (int32_t)L.size())) {
        g_parse_error = "arrays too small";
        *n_objs = (int32_t)O.size(); *n_mats = (int32_t)M.size(); *n_lights = (int32_t)L.size();
        return PPM_ERR_CAPACITY;
    }
    *n_objs = (int32_t)O.size();
    *n_mats = (int32_t)M.size();
    *n_lights = (int32_t)L.size();
    if (objs) std::memcpy(objs, O.data(), sizeof(ppm_object) * O.size());
    if (mats) std::memcpy(mats, M.data(), sizeof(ppm_material) * M.size());
    if (lights) std::memcpy(lights, L.data(), sizeof(ppm_light) * L.size());
    return PPM_OK;
}

extern "C" int ppm_camera_parse(const char *text, ppm_camera *cam, int64_t *nphoton) {
    g_parse_error.clear();
    if (!text || !cam) {
        g_parse_error = "null argument";
        return PPM_ERR_INVALID_ARG;
    }
    Doc d;
    if (!parse_doc(text, d)) return PPM_ERR_INVALID_ARG;
    // unset fields keep what the caller put in *cam (the reference camera's
    // values are a sensible start: ppm_camera of read_camera, camera.rs:108-146)
    const Entry &e = d.top;
    auto yesno = [&](const char *k, int32_t &out) -> bool {
        auto it = e.kv.find(k);
        if (it == e.kv.end()) return true;
        if (it->second == "yes") out = 1;
        else if (it->second == "no") out = 0;
        else return fail(e.line, std::string("'") + k + "' must be yes or no");
        return true;
    };
    auto num = [&](const char *k, double &out) -> bool {
        auto it = e.kv.find(k);
        if (it == e.kv.end()) return true;
        if (!to_num(it->second, out)) return fail(e.line, std::string("'") + k + "' is not a number");
        return true;
    };
    auto vec = [&](const char *k, double out[3]) -> bool {
        auto it = e.kv.find(k);
        if (it == e.kv.end()) return true;
        if (!to_vec(it->second, out)) return fail(e.line, std::string("'") + k + "' is not a vector");
        return true;
    };
    double xr = cam->xreso, yr = cam->yreso, ns = cam->n_sample_photon, np = nphoton ? (double)*nphoton : 0.0;
    double r = std::sqrt(cam->radius), focal_mm = cam->focal_len * 1000.0;
    if (!num("xresolution", xr) || !num("yresolution", yr) || !num("samplephoton", ns) || !num("nphoton", np) ||
        !yesno("progressive", cam->progressive) || !yesno("antialias", cam->antialias) ||
        !yesno("useclassic", cam->use_classic) || !yesno("blur", cam->blur) || !num("estimateradius", r) ||
        !num("maxradiance", cam->max_radiance) || !num("isosensitivity", cam->iso_sens) ||
        !num("shutterspeed", cam->shut_speed) || !num("focallength", focal_mm) || !num("fnumber", cam->f_number) ||
        !num("focus", cam->focus) || !vec("ambient", cam->ambient) || !vec("eyeposition", cam->eye_pos) ||
        !vec("targetposition", cam->target) || !vec("upperdirection", cam->upper))
        return PPM_ERR_INVALID_ARG;
    auto pf = e.kv.find("photonfilter");
    if (pf != e.kv.end()) {
        if (pf->second == "none") cam->pfilter = PPM_FILTER_NONE;
        else if (pf->second == "cone") cam->pfilter = PPM_FILTER_CONE;
        else if (pf->second == "gauss") cam->pfilter = PPM_FILTER_GAUSS;
        else return err(e.line, "photonfilter must be none, cone or gauss");
    }
    if (!(xr >= 1 && yr >= 1 && xr <= 65536 && yr <= 65536))
        return err(e.line, "resolution out of range");
    cam->xreso = (int32_t)xr;
    cam->yreso = (int32_t)yr;
    cam->n_sample_photon = (int32_t)ns;
    cam->radius = r * r;
    cam->focal_len = focal_mm / 1000.0;
    if (nphoton) *nphoton = (int64_t)np;
    ppm_camera_derive(cam);
    return PPM_OK;
}
