// rtc -- drop-in for the reference's classic ray tracer `rtc`
// (src/bin/rtc.rs): trace_ray_classic (tracer.rs:221-259) for every pixel,
// on the GPU (FP64) through the C ABI.
//
//   rtc <screen file> <scene file> [--passes N] [--seed S] [--read-files]
//
// Output as rtc.rs:24-40: the P3 header, then {:e} radiances if the camera is
// progressive, tone-mapped integers otherwise.  --passes N averages N
// anti-aliased passes.
#include "common.h"

int main(int argc, char **argv) {
    std::vector<std::string> args;
    unsigned long long seed = 1;
    int passes = 1;
    bool read_files = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--seed" && i + 1 < argc) seed = strtoull(argv[++i], nullptr, 10);
        else if (a == "--passes" && i + 1 < argc) passes = atoi(argv[++i]);
        else if (a == "--read-files") read_files = true;
        else args.push_back(a);
    }
    if (args.size() != 2 || passes < 1) {   // rtc.rs:20-24
        printf("Usage: rtc <screen file> <scene file>\n");
        return 0;
    }
    std::vector<ppm_object> objs;
    std::vector<ppm_material> mats;
    std::vector<ppm_light> lights;
    ppm_camera cam;
    if (!load_inputs(read_files, args[1], args[0], objs, mats, lights, cam, nullptr)) return 1;
    ppm_ctx *ctx = nullptr;
    if (ppm_ctx_create(&ctx, 0, seed)) { fprintf(stderr, "rtc: %s\n", ppm_last_error(nullptr)); return 1; }
    int st = ppm_scene_upload(ctx, objs.data(), (int)objs.size(), mats.data(), (int)mats.size(), lights.data(),
                              (int)lights.size());
    if (!st) st = ppm_camera_set(ctx, &cam);
    ppm_render_cfg cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.nphoton = 1;
    cfg.passes = passes;
    cfg.use_classic = 1;
    cfg.radius0 = 0.1;
    cfg.alpha = 0.5;
    cfg.schedule_offset = 1;
    cfg.precision = PPM_PRECISION_PLAIN;
    cfg.use_graph = 1;
    cfg.seed = seed;
    cfg.flags = PPM_RENDER_CLASSIC;
    std::vector<double> img((size_t)cam.xreso * cam.yreso * 3);
    if (!st) st = ppm_render(ctx, &cfg, img.data());
    if (st) {
        fprintf(stderr, "rtc: %s (%s)\n", ppm_status_string(st), ppm_last_error(ctx));
        ppm_ctx_destroy(ctx);
        return 1;
    }
    ppm_ctx_destroy(ctx);
    print_image(cam, img, !cam.progressive);
    return 0;
}
