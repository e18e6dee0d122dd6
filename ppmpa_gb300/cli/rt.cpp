// rt -- drop-in for the reference's eye-ray tracer `rt` (src/bin/rt.rs):
// reads a photon map in `pm`'s text format from standard input
// (photonmap.rs:31-74), builds it on the GPU and renders one eye pass
// (trace_ray for every pixel, FP64) through the C ABI.
//
//   rt <scene file> <camera file> [<radius>] [--seed S] [--read-files]
//
// Output as rt.rs:48-62: the P3 header, then {:e} radiances if the camera is
// progressive, tone-mapped integers (Camera::radiance_to_rgb) otherwise.
#include <iostream>

#include "common.h"

int main(int argc, char **argv) {
    std::vector<std::string> args;
    unsigned long long seed = 1;
    bool read_files = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--seed" && i + 1 < argc) seed = strtoull(argv[++i], nullptr, 10);
        else if (a == "--read-files") read_files = true;
        else args.push_back(a);
    }
    if (args.size() < 2) {   // rt.rs:22-27
        printf("Usage: rtc <scene file> <camera file> [<radius>]\n");
        return 0;
    }
    double radius2 = 0.1 * 0.1;
    if (args.size() == 3) {
        char *end = nullptr;
        double r = strtod(args[2].c_str(), &end);
        if (end != args[2].c_str() && !*end) radius2 = r * r;
    }
    std::vector<ppm_object> objs;
    std::vector<ppm_material> mats;
    std::vector<ppm_light> lights;
    ppm_camera cam;
    if (!load_inputs(read_files, args[0], args[1], objs, mats, lights, cam, nullptr)) return 1;
    // read_map (photonmap.rs:31-74): count line (ignored), power (1.0 if not a
    // number), then "Wl px py pz dx dy dz"; directions go through
    // Direction3::new_dir, i.e. are normalised
    std::string line;
    std::getline(std::cin, line);
    double power = 1.0;
    if (std::getline(std::cin, line)) {
        char *end = nullptr;
        std::string t = line;
        while (!t.empty() && isspace((unsigned char)t.back())) t.pop_back();
        double p = strtod(t.c_str(), &end);
        if (end != t.c_str() && !*end) power = p;
    }
    std::vector<double> pos, dir;
    std::vector<uint8_t> wl;
    while (std::getline(std::cin, line)) {
        if (line.empty()) continue;
        char name[16] = {0};
        double v[6];
        if (sscanf(line.c_str(), "%15s %lf %lf %lf %lf %lf %lf", name, v, v + 1, v + 2, v + 3, v + 4, v + 5) != 7) {
            fprintf(stderr, "rt: bad photon line: %s\n", line.c_str());
            return 1;
        }
        uint8_t w = strcmp(name, "Green") == 0 ? 1 : strcmp(name, "Blue") == 0 ? 2 : 0;
        double n = std::sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
        if (n == 0.0) { fprintf(stderr, "rt: zero photon direction\n"); return 1; }
        double inv = 1.0 / n;
        pos.insert(pos.end(), {v[0], v[1], v[2]});
        dir.insert(dir.end(), {v[3] * inv, v[4] * inv, v[5] * inv});
        wl.push_back(w);
    }
    ppm_ctx *ctx = nullptr;
    if (ppm_ctx_create(&ctx, 0, seed)) { fprintf(stderr, "rt: %s\n", ppm_last_error(nullptr)); return 1; }
    int st = ppm_scene_upload(ctx, objs.data(), (int)objs.size(), mats.data(), (int)mats.size(), lights.data(),
                              (int)lights.size());
    if (!st) st = ppm_camera_set(ctx, &cam);
    if (!st) st = ppm_photonmap_build(ctx, pos.data(), dir.data(), wl.data(), (int64_t)wl.size(), power, radius2);
    std::vector<double> img((size_t)cam.xreso * cam.yreso * 3);
    if (!st) st = ppm_eye_pass(ctx, 1, seed, 0, img.data());
    if (st) {
        fprintf(stderr, "rt: %s (%s)\n", ppm_status_string(st), ppm_last_error(ctx));
        ppm_ctx_destroy(ctx);
        return 1;
    }
    ppm_ctx_destroy(ctx);
    fprintf(stderr, "finished reading map: %zu photons.\n", wl.size());
    print_image(cam, img, !cam.progressive);
    return 0;
}
