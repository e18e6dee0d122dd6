// output.cpp -- the reference's image output stage on the host.
//
// ppm_tone_map: Camera::radiance_to_rgb (src/camera.rs:92-100) -- per channel
//   floor(min(1, L / max_radiance)^(1/2.2) * 255).  The averager applies the
//   same map to the average of its pass files (util/averager.rb:66-76), so
//   this also gives its P3 output from an averaged image.
// ppm_write_exr: the uncompressed scanline OpenEXR file util/averager2.rb
//   writes (header_exr / output_exr): channels B, G, R as 32-bit floats,
//   no compression, increasing-y line order, one line-offset table, then per
//   line its y, its byte count and the B, G and R rows; values are
//   L * scale (averager2.rb uses 1 / (passes * max radiance) on summed
//   images, i.e. 1 / max_radiance on an averaged one).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ppm_api.h"

namespace {

void put_u32(std::string &o, uint32_t v) {
    for (int k = 0; k < 4; k++) o += (char)((v >> (8 * k)) & 0xff);
}
void put_u64(std::string &o, uint64_t v) {
    for (int k = 0; k < 8; k++) o += (char)((v >> (8 * k)) & 0xff);
}
void put_f32(std::string &o, float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put_u32(o, u);
}
void put_str(std::string &o, const char *s) {
    o += s;
    o += '\0';
}
void put_attr(std::string &o, const char *name, const char *type, const std::string &value) {
    put_str(o, name);
    put_str(o, type);
    put_u32(o, (uint32_t)value.size());
    o += value;
}

}  // namespace

extern "C" int ppm_tone_map(const double *img, int64_t n, double max_radiance, int32_t *rgb_out) {
    if ((n && (!img || !rgb_out)) || n < 0 || !(max_radiance > 0.0)) return PPM_ERR_INVALID_ARG;
    const double gamma = 1.0 / 2.2;
    for (int64_t i = 0; i < n; i++) {
        double d = img[i] / max_radiance;
        double r = d > 1.0 ? 1.0 : d;
        rgb_out[i] = (int32_t)std::floor(std::pow(r, gamma) * 255.0);
    }
    return PPM_OK;
}

extern "C" int ppm_write_exr(const char *path, const double *img, int32_t xreso, int32_t yreso, double scale) {
    if (!path || !img || xreso <= 0 || yreso <= 0) return PPM_ERR_INVALID_ARG;
    std::string h;
    put_u32(h, 20000630u);   // magic
    put_u32(h, 2u);          // version 2, scanline
    std::string ch;
    for (const char *c : {"B", "G", "R"}) {
        put_str(ch, c);
        put_u32(ch, 2u);     // FLOAT
        put_u32(ch, 0u);     // pLinear, reserved
        put_u32(ch, 1u);     // xSampling
        put_u32(ch, 1u);     // ySampling
    }
    ch += '\0';
    put_attr(h, "channels", "chlist", ch);
    put_attr(h, "compression", "compression", std::string(1, '\0'));   // NO_COMPRESSION
    std::string box;
    for (uint32_t v : {0u, 0u, (uint32_t)(xreso - 1), (uint32_t)(yreso - 1)}) put_u32(box, v);
    put_attr(h, "dataWindow", "box2i", box);
    put_attr(h, "displayWindow", "box2i", box);
    put_attr(h, "lineOrder", "lineOrder", std::string(1, '\0'));       // INCREASING_Y
    std::string f1;
    put_f32(f1, 1.0f);
    put_attr(h, "pixelAspectRatio", "float", f1);
    std::string v2;
    put_f32(v2, 0.0f);
    put_f32(v2, 0.0f);
    put_attr(h, "screenWindowCenter", "v2f", v2);
    put_attr(h, "screenWindowWidth", "float", f1);
    h += '\0';
    const uint64_t datalen = 4ull * (uint64_t)xreso * 3ull;
    const uint64_t linelen = 8ull + datalen;
    const uint64_t first = (uint64_t)h.size() + 8ull * (uint64_t)yreso;
    std::string body;
    body.reserve((size_t)(8ull * yreso + linelen * yreso));
    for (int32_t y = 0; y < yreso; y++) put_u64(body, first + linelen * (uint64_t)y);
    for (int32_t y = 0; y < yreso; y++) {
        put_u32(body, (uint32_t)y);
        put_u32(body, (uint32_t)datalen);
        for (int c = 2; c >= 0; c--)   // B, G, R rows
            for (int32_t x = 0; x < xreso; x++)
                put_f32(body, (float)(img[3 * ((size_t)y * xreso + x) + c] * scale));
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) return PPM_ERR_INVALID_ARG;
    bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size() && std::fwrite(body.data(), 1, body.size(), f) == body.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? PPM_OK : PPM_ERR_INVALID_ARG;
}
