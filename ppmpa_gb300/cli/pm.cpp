// pm -- drop-in for the reference's photon tracer `pm` (src/bin/pm.rs),
// tracing on the GPU (FP64, the reference's arithmetic) through the C ABI.
//
//   pm [-c|-h] <scene file> [<#photon>] [--seed S] [--read-files]
//
// Prints the photon map in the reference's text format (pm.rs:44-45,
// :62-75): the photon count, the photon power, then one line per stored
// photon, "Red|Green|Blue px py pz dx dy dz" in Rust's {} format, lights in
// scene order, each emitted photon's stored photons deepest bounce first
// (the order trace_photon returns them).  `rt` reads this format.
#include <algorithm>
#include <numeric>

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
    // pm.rs:21-37
    if (args.empty() || args[0] == "-h") {
        printf("Usage: pm [-c|-h] <scene file> [<#photon>] (output photon map to stdout)\n");
        return 0;
    }
    long long nphoton = 100000;
    if (args.size() == 2) {
        char *end = nullptr;
        long long n = strtoll(args[1].c_str(), &end, 10);
        if (end != args[1].c_str() && !*end && n >= -2147483648LL && n <= 2147483647LL) nphoton = n;
    }
    std::vector<ppm_object> objs;
    std::vector<ppm_material> mats;
    std::vector<ppm_light> lights;
    ppm_camera cam;
    if (!load_inputs(read_files, args[0], "", objs, mats, lights, cam, nullptr)) return 1;
    ppm_ctx *ctx = nullptr;
    if (ppm_ctx_create(&ctx, 0, seed)) { fprintf(stderr, "pm: %s\n", ppm_last_error(nullptr)); return 1; }
    int64_t n_stored = 0, n_emitted = 0;
    double power = 0.0;
    int st = ppm_scene_upload(ctx, objs.data(), (int)objs.size(), mats.data(), (int)mats.size(), lights.data(),
                              (int)lights.size());
    if (!st) st = ppm_trace_photons(ctx, nphoton, 1, 0, &n_stored, &power, &n_emitted);
    std::vector<double> pos(3 * (size_t)n_stored), dir(3 * (size_t)n_stored);
    std::vector<uint8_t> wl((size_t)n_stored);
    std::vector<int32_t> emit((size_t)n_stored);
    std::vector<int8_t> level((size_t)n_stored);
    if (!st) st = ppm_photons_download(ctx, pos.data(), dir.data(), wl.data(), emit.data(), level.data(), n_stored);
    if (st) {
        fprintf(stderr, "pm: %s (%s)\n", ppm_status_string(st), ppm_last_error(ctx));
        ppm_ctx_destroy(ctx);
        return 1;
    }
    ppm_ctx_destroy(ctx);
    std::vector<size_t> order((size_t)n_stored);
    std::iota(order.begin(), order.end(), (size_t)0);
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return emit[a] != emit[b] ? emit[a] < emit[b] : level[a] > level[b];
    });
    printf("%lld\n%s\n", nphoton, rust_display(power).c_str());
    const char *names[3] = {"Red", "Green", "Blue"};
    for (size_t k : order)
        printf("%s %s %s %s %s %s %s\n", names[wl[k] % 3], rust_display(pos[3 * k]).c_str(),
               rust_display(pos[3 * k + 1]).c_str(), rust_display(pos[3 * k + 2]).c_str(),
               rust_display(dir[3 * k]).c_str(), rust_display(dir[3 * k + 1]).c_str(),
               rust_display(dir[3 * k + 2]).c_str());
    return 0;
}
