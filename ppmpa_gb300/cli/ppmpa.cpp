// ppmpa -- command-line drop-in for the reference's `ppmpa` binary
// (src/bin/ppmpa.rs), running the pass on the GPU through the C ABI.
//
//   ppmpa [-nc|-h] <#photon> <radius> <camera file> <scene file>
//         [--passes N] [--alpha A] [--seed S] [--plain] [--read-files]
//         [--ppm] [--exr FILE]
//
// Without --passes it renders one pass, like the reference binary
// (ppmpa.rs:74-84), and prints the P3 header of Camera::pnm_header
// (camera.rs:77-90) followed by one "r g b" line per pixel in Rust's {:e}
// format (camera.rs:212-214).  The reference ignores its camera and scene
// file arguments and uses the built-in scene (scene.rs:20-448) and camera
// defaults (camera.rs:108-206); so does this program.  With --passes N it
// runs the progressive loop on the GPU (radius schedule of util/iterator.rb,
// average of util/averager.rb) and prints the averaged image.
// --read-files reads the scene and camera files (ppm_scene_parse /
// ppm_camera_parse) instead; --ppm prints tone-mapped integers like the
// averager; --exr also writes the averager2 OpenEXR file.
#include "common.h"

namespace {

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
    bool read_files = false, integers = false;
    std::string exr;
    for (size_t i = 1; i < args.size(); i++) {
        if (args[i] == "--passes" && i + 1 < args.size()) passes = atoi(args[++i].c_str());
        else if (args[i] == "--alpha" && i + 1 < args.size()) alpha = atof(args[++i].c_str());
        else if (args[i] == "--seed" && i + 1 < args.size()) seed = strtoull(args[++i].c_str(), nullptr, 10);
        else if (args[i] == "--plain") precision = PPM_PRECISION_PLAIN;
        else if (args[i] == "--read-files") read_files = true;
        else if (args[i] == "--ppm") integers = true;
        else if (args[i] == "--exr" && i + 1 < args.size()) exr = args[++i];
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
    ppm_camera cam;
    if (!load_inputs(read_files, pos[off + 3], pos[off + 2], objs, mats, lights, cam, nullptr)) return 1;

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

    if (!exr.empty() && ppm_write_exr(exr.c_str(), img.data(), cam.xreso, cam.yreso, 1.0 / cam.max_radiance)) {
        fprintf(stderr, "ppmpa: cannot write %s\n", exr.c_str());
        return 1;
    }
    print_image(cam, img, integers);
    return 0;
}
