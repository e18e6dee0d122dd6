// ppmpa -- command-line drop-in for the reference's `ppmpa` binary
// (src/bin/ppmpa.rs), running the pass on the GPU through the C ABI.
//
//   ppmpa [-nc|-h] <#photon> <radius> <camera file> <scene file>
//         [--passes N] [--alpha A] [--seed S] [--plain]
//
// Without --passes it renders one pass, like the reference binary
// (ppmpa.rs:74-84), and prints the P3 header of Camera::pnm_header
// (camera.rs:77-90) followed by one "r g b" line per pixel in Rust's {:e}
// format (camera.rs:212-214).  The reference ignores its camera and scene
// file arguments and uses the built-in scene (scene.rs:20-448) and camera
// defaults (camera.rs:108-206); so does this program.  With --passes N it
// runs the progressive loop on the GPU (radius schedule of util/iterator.rb,
// average of util/averager.rb) and prints the averaged image.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
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

int usage() {
    fprintf(stderr, "Usage: ppmpa [-nc|-h] <#photon> <radius> <camera file> <scene file>\n");
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    std::vector<std::string> args(argv, argv + argc);
    if (args.size() > 1 && args[1] == "--format-test") {   // prints {:e} and {} of each value
        for (size_t i = 2; i < args.size(); i++) {
            double v = strtod(args[i].c_str(), nullptr);
            printf("%s %s\n", rust_lower_exp(v).c_str(), rust_display(v).c_str());
        }
        return 0;
    }
    // ppmpa.rs:21-27: fewer than 4 positional arguments or -h prints the usage
    std::vector<std::string> pos;
    int passes = 0;
    double alpha = 0.5;
    unsigned long long seed = 1;
    int precision = PPM_PRECISION_MIXED;
    for (size_t i = 1; i < args.size(); i++) {
        if (args[i] == "--passes" && i + 1 < args.size()) passes = atoi(args[++i].c_str());
        else if (args[i] == "--alpha" && i + 1 < args.size()) alpha = atof(args[++i].c_str());
        else if (args[i] == "--seed" && i + 1 < args.size()) seed = strtoull(args[++i].c_str(), nullptr, 10);
        else if (args[i] == "--plain") precision = PPM_PRECISION_PLAIN;
        else pos.push_back(args[i]);
    }
    if (pos.size() < 4 || pos[0] == "-h") return usage();
    size_t off = 0;
    bool uc = true;
    if (pos[0] == "-nc") { off = 1; uc = false; }       // ppmpa.rs:50-54
    if (pos.size() < off + 4) return usage();
    // ppmpa.rs:56-63: unparsable values fall back to the defaults
    char *end = nullptr;
    long long nphoton = strtoll(pos[off].c_str(), &end, 10);
    if (end == pos[off].c_str() || *end) nphoton = 100000;
    double radius = strtod(pos[off + 1].c_str(), &end);
    if (end == pos[off + 1].c_str() || *end) radius = 0.1;

    std::vector<ppm_object> objs;
    std::vector<ppm_material> mats;
    std::vector<ppm_light> lights;
    reference_scene(objs, mats, lights);
    ppm_camera cam = reference_camera();

    ppm_ctx *ctx = nullptr;
    int st = ppm_ctx_create(&ctx, 0, seed);
    if (st) { fprintf(stderr, "ppmpa: %s\n", ppm_last_error(nullptr)); return 1; }
    st = ppm_scene_upload(ctx, objs.data(), (int)objs.size(), mats.data(), (int)mats.size(), lights.data(),
                          (int)lights.size());
    if (!st) st = ppm_camera_set(ctx, &cam);
    ppm_render_cfg cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.nphoton = nphoton;
    cfg.passes = passes > 0 ? passes : 1;
    cfg.use_classic = uc ? 1 : 0;
    cfg.radius0 = radius;
    cfg.alpha = alpha;
    cfg.schedule_offset = 1;
    cfg.precision = precision;
    cfg.use_graph = 1;
    cfg.seed = seed;
    std::vector<double> img((size_t)cam.xreso * cam.yreso * 3);
    if (!st) st = ppm_render(ctx, &cfg, img.data());
    if (st) {
        fprintf(stderr, "ppmpa: %s (%s)\n", ppm_status_string(st), ppm_last_error(ctx));
        ppm_ctx_destroy(ctx);
        return 1;
    }
    ppm_ctx_destroy(ctx);

    // Camera::pnm_header (camera.rs:77-90)
    std::string ss = cam.shut_speed < 1.0 ? "1/" + rust_display(1.0 / cam.shut_speed) : rust_display(cam.shut_speed);
    printf("P3\n## max radiance = %s\n## image parameters = %s, F%s, ISO%s\n%d %d\n255\n",
           rust_display(cam.max_radiance).c_str(), ss.c_str(), rust_display(cam.f_number).c_str(),
           rust_display(cam.iso_sens).c_str(), cam.xreso, cam.yreso);
    for (size_t p = 0; p < (size_t)cam.xreso * cam.yreso; p++)
        printf("%s %s %s\n", rust_lower_exp(img[3 * p]).c_str(), rust_lower_exp(img[3 * p + 1]).c_str(),
               rust_lower_exp(img[3 * p + 2]).c_str());
    return 0;
}
