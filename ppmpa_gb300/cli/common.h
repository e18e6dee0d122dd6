// common.h -- pieces shared by the ppmpa, pm and rt programs: Rust's f64
// formatting, the reference's built-in scene and camera, scene/camera file
// loading, and the P3 output of Camera::pnm_header (src/camera.rs:77-90).
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ppm_api.h"

namespace {

// Rust's f64 formatting prints the shortest decimal that round-trips.
std::string shortest_digits(double v, int &exp10) {
    char buf[64];
    for (int prec = 0; prec <= 17; prec++) {
        snprintf(buf, sizeof buf, "%.*e", prec, v);
        if (strtod(buf, nullptr) == v) break;
    }
    // buf = "d.ddde[+-]xx"
    std::string s(buf);
    size_t e = s.find('e');
    exp10 = atoi(s.c_str() + e + 1);
    std::string mant = s.substr(0, e);
    std::string digits;
    for (char c : mant)
        if (c >= '0' && c <= '9') digits += c;
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    return digits;
}

// format!("{:e}", v) for finite v: "1.234e-3", "0e0", "5e-1"
std::string rust_lower_exp(double v) {
    if (v == 0.0) return std::signbit(v) ? "-0e0" : "0e0";
    std::string sign = v < 0 ? "-" : "";
    int e;
    std::string d = shortest_digits(std::fabs(v), e);
    std::string out = sign + d.substr(0, 1);
    if (d.size() > 1) out += "." + d.substr(1);
    return out + "e" + std::to_string(e);
}

// format!("{}", v) for f64: shortest round-trip digits, positional notation
std::string rust_display(double v) {
    if (v == 0.0) return "0";
    std::string sign = v < 0 ? "-" : "";
    int e;
    std::string d = shortest_digits(std::fabs(v), e);
    std::string out;
    int point = e + 1;   // digits before the decimal point
    if (point <= 0) {
        out = "0." + std::string(-point, '0') + d;
    } else if ((size_t)point >= d.size()) {
        out = d + std::string(point - d.size(), '0');
    } else {
        out = d.substr(0, point) + "." + d.substr(point);
    }
    return sign + out;
}

void v3(double *dst, double x, double y, double z) { dst[0] = x; dst[1] = y; dst[2] = z; }

ppm_material simple(double r, double g, double b, double sr, double sg, double sb, double diff, double meta,
                    double rough) {
    ppm_material m;
    memset(&m, 0, sizeof m);
    m.surface = PPM_SURF_SIMPLE;
    v3(m.color_diff, r, g, b);
    v3(m.color_spec, sr, sg, sb);
    m.scatter = diff;
    m.metalness = meta;
    m.roughness = rough;
    ppm_material_derive(&m);
    return m;
}

ppm_material ts(double r, double g, double b, double sr, double sg, double sb, double scat, double meta, double rough) {
    ppm_material m = simple(r, g, b, sr, sg, sb, scat, meta, rough);
    m.surface = PPM_SURF_TS;
    ppm_material_derive(&m);
    return m;
}

ppm_object plain(double nx, double ny, double nz, double d, int mat) {
    ppm_object o;
    memset(&o, 0, sizeof o);
    o.shape = PPM_SHAPE_PLAIN;
    o.material = mat;
    v3(o.nvec, nx, ny, nz);
    o.dist = d;
    return o;
}

ppm_object sphere(double x, double y, double z, double r, int mat) {
    ppm_object o;
    memset(&o, 0, sizeof o);
    o.shape = PPM_SHAPE_SPHERE;
    o.material = mat;
    v3(o.position, x, y, z);
    o.radius = r;
    return o;
}

// read_scene (src/scene.rs:20-448) as data
void reference_scene(std::vector<ppm_object> &objs, std::vector<ppm_material> &mats, std::vector<ppm_light> &lights) {
    ppm_light l;
    memset(&l, 0, sizeof l);
    l.kind = PPM_LIGHT_PARALLELOGRAM;
    v3(l.color, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0);   // Color(1,1,1).normalize()
    l.flux = 5.0;
    v3(l.pos, -0.67, 3.99, 2.33);
    v3(l.nvec, -0.0, -1.0, -0.0);
    v3(l.dir1, 1.33, 0.0, 0.0);
    v3(l.dir2, 0.0, 0.0, 1.33);
    lights.push_back(l);
    mats.push_back(simple(0.5, 0.5, 0.5, 0.8, 0.8, 0.8, 1.0, 0.0, 0.0));     // 0 mwall
    mats.push_back(simple(0.1, 0.1, 0.4, 0.8, 0.0, 0.8, 1.0, 0.0, 0.0));     // 1 mwallb
    mats.push_back(simple(0.4, 0.1, 0.1, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0));     // 2 mwallr
    ppm_material b10 = ts(1.0, 1.0, 1.0, 0.05, 0.05, 0.05, 0.0, 0.0, 0.8);
    v3(b10.ior, 1.5, 1.5, 1.5);
    mats.push_back(b10);                                                      // 3 ball10
    mats.push_back(simple(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.9));  // 4 ball9
    mats.push_back(simple(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.8));  // 5 ball8
    mats.push_back(simple(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.7));  // 6 ball7
    mats.push_back(ts(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.6));      // 7 ball6
    mats.push_back(ts(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.5));      // 8 ball5
    mats.push_back(simple(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.4));  // 9 ball4
    mats.push_back(simple(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.3));  // 10 ball3
    mats.push_back(simple(0.0, 0.0, 0.0, 0.78, 0.78, 0.78, 0.0, 1.0, 0.2));  // 11 ball2
    ppm_material b1 = ts(0.6, 0.35, 0.1, 0.05, 0.05, 0.05, 1.0, 0.0, 0.0);
    v3(b1.ior, 1.5, 1.5, 1.5);
    mats.push_back(b1);                                                       // 12 ball1
    ppm_material mp = simple(0.0, 0.0, 0.0, 0.8, 0.8, 0.8, 0.0, 0.0, 0.0);
    v3(mp.emittance, 0.15, 0.15, 0.15);
    mats.push_back(mp);                                                       // 13 mparal
    objs.push_back(plain(0.0, 1.0, 0.0, 0.0, 0));
    objs.push_back(plain(-0.0, -1.0, -0.0, 4.0, 0));
    objs.push_back(plain(-1.0, -0.0, -0.0, 2.0, 1));
    objs.push_back(plain(1.0, 0.0, 0.0, 2.0, 2));
    objs.push_back(plain(0.0, 0.0, 1.0, 6.0, 0));
    objs.push_back(plain(-0.0, -0.0, -1.0, 5.0, 0));
    const double xs[5] = {-1.6, -0.8, 0.0, 0.8, 1.6};
    const int top[5] = {12, 11, 10, 9, 8}, bottom[5] = {7, 6, 5, 4, 3};
    for (int i = 0; i < 5; i++) objs.push_back(sphere(xs[i], 1.5, 3.0, 0.4, top[i]));
    for (int i = 0; i < 5; i++) objs.push_back(sphere(xs[i], 0.5, 2.5, 0.4, bottom[i]));
    ppm_object panel;
    memset(&panel, 0, sizeof panel);
    panel.shape = PPM_SHAPE_PARALLELOGRAM;
    panel.material = 13;
    v3(panel.position, -0.67, 3.99, 2.33);
    v3(panel.nvec, -0.0, -1.0, -0.0);
    v3(panel.dir1, 0.67 - -0.67, 3.99 - 3.99, 2.33 - 2.33);
    v3(panel.dir2, -0.67 - -0.67, 3.99 - 3.99, 3.67 - 2.33);
    objs.push_back(panel);
}

// read_camera defaults (src/camera.rs:108-146)
ppm_camera reference_camera() {
    ppm_camera c;
    memset(&c, 0, sizeof c);
    c.xreso = 256;
    c.yreso = 256;
    c.progressive = 1;
    c.antialias = 1;
    c.use_classic = 1;
    c.blur = 1;
    c.radius = 0.2 * 0.2;
    c.max_radiance = 0.01;
    c.iso_sens = 100.0;
    c.shut_speed = 0.004;
    c.focal_len = 50.0 / 1000.0;
    c.f_number = 4.0;
    c.focus = 7.0;
    c.pfilter = PPM_FILTER_NONE;
    c.n_sample_photon = 500;
    v3(c.eye_pos, 1.0, 2.0, -4.5);
    v3(c.target, 0.0, 1.0, 0.0);
    v3(c.upper, 0.0, 1.0, 0.0);
    ppm_camera_derive(&c);
    return c;
}

// The reference ignores its scene and camera file arguments (scene.rs:20,
// camera.rs:108); with read_files the programs parse them instead.
inline bool load_inputs(bool read_files, const std::string &scene_file, const std::string &camera_file,
                        std::vector<ppm_object> &objs, std::vector<ppm_material> &mats,
                        std::vector<ppm_light> &lights, ppm_camera &cam, long long *nphoton) {
    cam = reference_camera();
    if (!read_files) {
        reference_scene(objs, mats, lights);
        return true;
    }
    auto slurp = [](const std::string &path, std::string &out) {
        std::ifstream f(path, std::ios::binary);
        if (!f) return false;
        std::stringstream ss;
        ss << f.rdbuf();
        out = ss.str();
        return true;
    };
    std::string text;
    if (!scene_file.empty()) {
        if (!slurp(scene_file, text)) { fprintf(stderr, "cannot read %s\n", scene_file.c_str()); return false; }
        int32_t no = 0, nm = 0, nl = 0;
        if (ppm_scene_parse(text.c_str(), nullptr, &no, nullptr, &nm, nullptr, &nl)) {
            fprintf(stderr, "%s: %s\n", scene_file.c_str(), ppm_parse_error());
            return false;
        }
        objs.resize(no); mats.resize(nm); lights.resize(nl);
        if (ppm_scene_parse(text.c_str(), objs.data(), &no, mats.data(), &nm, lights.data(), &nl)) {
            fprintf(stderr, "%s: %s\n", scene_file.c_str(), ppm_parse_error());
            return false;
        }
    } else {
        reference_scene(objs, mats, lights);
    }
    if (!camera_file.empty()) {
        if (!slurp(camera_file, text)) { fprintf(stderr, "cannot read %s\n", camera_file.c_str()); return false; }
        int64_t np = nphoton ? *nphoton : 0;
        if (ppm_camera_parse(text.c_str(), &cam, &np)) {
            fprintf(stderr, "%s: %s\n", camera_file.c_str(), ppm_parse_error());
            return false;
        }
        if (nphoton) *nphoton = np;
    }
    return true;
}

// Camera::pnm_header (camera.rs:77-90), then one line per pixel: "{:e}"
// radiances (progressive, camera.rs:212-214) or tone-mapped integers
// (camera.rs:92-100, 208-210)
inline void print_image(const ppm_camera &cam, const std::vector<double> &img, bool integers) {
    std::string ss = cam.shut_speed < 1.0 ? "1/" + rust_display(1.0 / cam.shut_speed) : rust_display(cam.shut_speed);
    printf("P3\n## max radiance = %s\n## image parameters = %s, F%s, ISO%s\n%d %d\n255\n",
           rust_display(cam.max_radiance).c_str(), ss.c_str(), rust_display(cam.f_number).c_str(),
           rust_display(cam.iso_sens).c_str(), cam.xreso, cam.yreso);
    const size_t npx = (size_t)cam.xreso * cam.yreso;
    if (integers) {
        std::vector<int32_t> rgb(3 * npx);
        ppm_tone_map(img.data(), (int64_t)(3 * npx), cam.max_radiance, rgb.data());
        for (size_t p = 0; p < npx; p++) printf("%d %d %d\n", rgb[3 * p], rgb[3 * p + 1], rgb[3 * p + 2]);
        return;
    }
    for (size_t p = 0; p < npx; p++)
        printf("%s %s %s\n", rust_lower_exp(img[3 * p]).c_str(), rust_lower_exp(img[3 * p + 1]).c_str(),
               rust_lower_exp(img[3 * p + 2]).c_str());
}

}  // namespace
