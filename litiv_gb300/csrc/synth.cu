// Seeded synthetic scenes (include/lvbgs_synth.h). All arithmetic is integer so the host and the
// device renderers agree byte for byte; the only floating-point values (ripple and drift tables,
// Gaussian weights) are computed once on the host and shared.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/lvbgs_synth.h"
#include "lvbgs_internal.h"

using namespace lvbgs;

namespace {

constexpr int kRippleW = 400, kRippleH = 300, kRipplePeriod = 407;  // 2*pi*(x/37 + t/11) = 2*pi*(11x+37t)/407

struct Shape {
    int x, y, w, h;  // position of this frame (top-left), size
    int ellipse;
    uint32_t col;  // packed channel values
};
constexpr int kFalloffN = 1024;  // falloff table over u = 256 * d^2 / r^2 in [0, 4)
struct FrameParams {
    int W, H, C;
    int nShapes;
    int thermal;  // shapes are blobs: (x, y) centre, w radius, col intensity
    Shape shapes[LVSYNTH_MAX_SHAPES];
    int drift;
    int rippleOn, rx0, ry0;
    uint32_t t;
    uint64_t seed;
    int sigmaMilli;
};

uint32_t rnd32(uint64_t seed, uint32_t a, uint32_t b, uint32_t c, int lane) {
    uint32_t ctr[4] = {a, b, c, 0x5EEDu};
    philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
    return ctr[lane & 3];
}
int rnd_range(uint64_t seed, uint32_t a, uint32_t b, int lo, int hi) {  // [lo, hi]
    if (hi <= lo) return lo;
    return lo + (int)(rnd32(seed, a, b, 0x51u, 0) % (uint32_t)(hi - lo + 1));
}

LV_HD int reflect_pos(long long p, long long range) {
    if (range <= 0) return 0;
    const long long period = 2 * range;
    long long m = p % period;
    if (m < 0) m += period;
    if (m > range) m = period - m;
    return (int)(m >> 8);
}

// one pixel of frame t (host and device)
LV_HD void render_px(const FrameParams& F, const uint8_t* tex, const int8_t* rippleTab, const uint16_t* falloff, int x,
                     int y, uint8_t* out, uint8_t* gt) {
    const int C = F.C;
    int v[3];
    const size_t p = (size_t)y * F.W + x;
    for (int c = 0; c < C; ++c) v[c] = tex[p * C + c] + F.drift;
    int inside = 0;
    if (F.thermal) {
        // warm blobs with a Gaussian falloff: v += (I - v) * f(d^2 / r^2), f in 1/256
        for (int i = 0; i < F.nShapes; ++i) {
            const Shape& s = F.shapes[i];
            const long long dx = x - s.x, dy = y - s.y, r2 = (long long)s.w * s.w;
            const long long d2 = dx * dx + dy * dy;
            if (d2 >= 4 * r2) continue;
            const int f = falloff[(int)(d2 * 256 / r2)];
            for (int c = 0; c < C; ++c) v[c] += (int)(((long long)((int)s.col - v[c]) * f) / 256);
            if (d2 < r2) inside = 1;
        }
    }
    if (F.rippleOn && x >= F.rx0 && x < F.rx0 + kRippleW && y >= F.ry0 && y < F.ry0 + kRippleH) {
        const int r = rippleTab[(int)((11u * (uint32_t)x + 37u * F.t) % (uint32_t)kRipplePeriod)];
        for (int c = 0; c < C; ++c) v[c] += r;
    }
    for (int i = 0; i < (F.thermal ? 0 : F.nShapes); ++i) {
        const Shape& s = F.shapes[i];
        const int dx = x - s.x, dy = y - s.y;
        if (dx < 0 || dy < 0 || dx >= s.w || dy >= s.h) continue;
        bool in = true;
        if (s.ellipse) {
            // (2dx+1-w)^2 * h^2 + (2dy+1-h)^2 * w^2 <= w^2 h^2
            const long long ex = 2 * dx + 1 - s.w, ey = 2 * dy + 1 - s.h;
            const long long w2 = (long long)s.w * s.w, h2 = (long long)s.h * s.h;
            in = ex * ex * h2 + ey * ey * w2 <= w2 * h2;
        }
        if (in) {
            inside = 1;
            for (int c = 0; c < C; ++c) v[c] = (int)((s.col >> (8 * c)) & 0xffu);
        }
    }
    // noise: Irwin-Hall sum of 4 uniform bytes (mean 510, sd 147.801) scaled to sigma
    uint32_t ctr[4] = {(uint32_t)p, F.t, 0x0015Eu, 0u};
    philox4x32_10(ctr, (uint32_t)F.seed, (uint32_t)(F.seed >> 32));
    for (int c = 0; c < C; ++c) {
        const uint32_t r = ctr[c];
        const int sum = (int)(r & 0xffu) + (int)((r >> 8) & 0xffu) + (int)((r >> 16) & 0xffu) + (int)(r >> 24);
        const long long n = (long long)(sum - 510) * F.sigmaMilli / 147801;
        int o = v[c] + (int)n;
        out[p * C + c] = (uint8_t)(o < 0 ? 0 : o > 255 ? 255 : o);
    }
    if (gt) gt[p] = inside ? 255 : 0;
}

__global__ void render_kernel(FrameParams F, const uint8_t* tex, const int8_t* rippleTab, const uint16_t* falloff,
                              uint8_t* out, uint8_t* gt) {
    const int total = F.W * F.H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x)
        render_px(F, tex, rippleTab, falloff, p % F.W, p / F.W, out, gt);
}

}  // namespace

struct lvsynth_scene {
    lvsynth_config cfg;
    std::vector<uint8_t> tex;
    int8_t ripple[kRipplePeriod];
    int rx0 = 0, ry0 = 0;
    struct ShapeInit {
        int w, h, ellipse;
        uint32_t col;
        long long x0, y0, vx, vy;  // 1/256 px
        int tstop;
    } shapes[LVSYNTH_MAX_SHAPES];
    uint16_t falloff[kFalloffN];
    uint8_t* d_tex = nullptr;
    int8_t* d_ripple = nullptr;
    uint16_t* d_falloff = nullptr;
};

namespace {

// thermal background: diagonal gradient 80..140 plus value noise of amplitude 10 on a 64-px grid
void build_thermal_texture(lvsynth_scene* s) {
    const int W = s->cfg.width, H = s->cfg.height, C = s->cfg.channels;
    const uint64_t seed = s->cfg.seed;
    const int G = 64, gw = W / G + 2, gh = H / G + 2;
    std::vector<int> grid((size_t)gw * gh);
    for (int j = 0; j < gh; ++j)
        for (int i = 0; i < gw; ++i) grid[(size_t)j * gw + i] = rnd_range(seed, 0x7E0u + (uint32_t)j, (uint32_t)i, -10, 10);
    s->tex.resize((size_t)W * H * C);
    const long long span = (long long)(W + H - 2 > 0 ? W + H - 2 : 1);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const int gx = x / G, gy = y / G, fx = x % G, fy = y % G;
            const long long a = grid[(size_t)gy * gw + gx], b = grid[(size_t)gy * gw + gx + 1];
            const long long c = grid[(size_t)(gy + 1) * gw + gx], d = grid[(size_t)(gy + 1) * gw + gx + 1];
            const long long top = a * (G - fx) + b * fx, bot = c * (G - fx) + d * fx;
            const long long vn = top * (G - fy) + bot * fy;  // value noise x 64*64
            const long long grad = 80 * 4096 + 60 * 4096 * (long long)(x + y) / span;
            const long long v = (grad + vn + (vn >= 0 ? 2048 : -2048)) / 4096;
            for (int ch = 0; ch < C; ++ch) s->tex[((size_t)y * W + x) * C + ch] = (uint8_t)std::min<long long>(std::max<long long>(v, 0), 255);
        }
}

void build_texture(lvsynth_scene* s) {
    const int W = s->cfg.width, H = s->cfg.height, C = s->cfg.channels;
    const uint64_t seed = s->cfg.seed;
    // Gaussian weights, sigma 4, radius 12, integer, summing to 65536
    const int R = 12;
    int wts[2 * R + 1];
    double g[2 * R + 1], gs = 0;
    for (int i = -R; i <= R; ++i) gs += (g[i + R] = std::exp(-(double)(i * i) / (2.0 * 16.0)));
    int tot = 0;
    for (int i = 0; i < 2 * R + 1; ++i) tot += (wts[i] = (int)std::lround(65536.0 * g[i] / gs));
    wts[R] += 65536 - tot;
    const size_t n = (size_t)W * H * C;
    std::vector<uint8_t> u(n);
    for (size_t i = 0; i < n; i += 4) {
        uint32_t ctr[4] = {(uint32_t)(i >> 2), (uint32_t)(i >> 34), 0x7E47u, 0u};
        philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (size_t k = 0; k < 4 && i + k < n; ++k) u[i + k] = (uint8_t)(ctr[k] & 0xffu);
    }
    std::vector<uint32_t> hpass(n);
    const int nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    auto run_rows = [&](auto fn) {
        std::vector<std::thread> th;
        for (int k = 0; k < nth; ++k) th.emplace_back([&, k] {
            for (int y = k; y < H; y += nth) fn(y);
        });
        for (auto& t : th) t.join();
    };
    run_rows([&](int y) {
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) {
                uint32_t acc = 0;
                for (int i = -R; i <= R; ++i) {
                    const int xx = std::min(std::max(x + i, 0), W - 1);
                    acc += (uint32_t)wts[i + R] * u[((size_t)y * W + xx) * C + c];
                }
                hpass[((size_t)y * W + x) * C + c] = acc;
            }
    });
    s->tex.resize(n);
    run_rows([&](int y) {
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) {
                uint64_t acc = 0;
                for (int i = -R; i <= R; ++i) {
                    const int yy = std::min(std::max(y + i, 0), H - 1);
                    acc += (uint64_t)wts[i + R] * hpass[((size_t)yy * W + x) * C + c];
                }
                const int sm = (int)((acc + (1ull << 31)) >> 32);
                const int v = 128 + (sm - 128) * 6;
                s->tex[((size_t)y * W + x) * C + c] = (uint8_t)std::min(std::max(v, 0), 255);
            }
    });
}

FrameParams frame_params(const lvsynth_scene* s, int t) {
    FrameParams F;
    std::memset(&F, 0, sizeof(F));
    const lvsynth_config& c = s->cfg;
    F.W = c.width;
    F.H = c.height;
    F.C = c.channels;
    F.t = (uint32_t)t;
    F.seed = c.seed;
    F.sigmaMilli = c.noise_sigma_milli;
    F.drift = c.drift ? (int)std::lround(15.0 * std::sin(2.0 * M_PI * t / 250.0)) : 0;
    F.rippleOn = c.ripple;
    F.rx0 = s->rx0;
    F.ry0 = s->ry0;
    F.nShapes = c.n_shapes;
    F.thermal = c.thermal;
    if (c.thermal) {
        // random walks: step k of blob i is one of eight directions times a length in [speed_min, speed_max]
        static const int dirs[8][2] = {{1, 0}, {1, 1}, {0, 1}, {-1, 1}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}};
        for (int i = 0; i < c.n_shapes; ++i) {
            const auto& si = s->shapes[i];
            long long px = si.x0, py = si.y0;
            const int r = si.w;
            for (int k = 0; k < t; ++k) {
                const uint32_t rr = rnd32(c.seed, 0xB10Bu + (uint32_t)i, (uint32_t)k, 0x57u, 0);
                const int dir = (int)(rr & 7u);
                const int len = c.speed_min_q8 + (int)((rr >> 3) % (uint32_t)(c.speed_max_q8 - c.speed_min_q8 + 1));
                px += dirs[dir][0] * len;
                py += dirs[dir][1] * len;
                // reflect into [r, W-1-r] x [r, H-1-r]
                const long long lx = r, hx = c.width - 1 - r, ly = r, hy = c.height - 1 - r;
                if (hx > lx) {
                    while (px < lx || px > hx) px = px < lx ? 2 * lx - px : 2 * hx - px;
                } else {
                    px = c.width / 2;
                }
                if (hy > ly) {
                    while (py < ly || py > hy) py = py < ly ? 2 * ly - py : 2 * hy - py;
                } else {
                    py = c.height / 2;
                }
            }
            Shape& o = F.shapes[i];
            o.x = (int)px;
            o.y = (int)py;
            o.w = r;
            o.h = r;
            o.ellipse = 1;
            o.col = si.col;
        }
        return F;
    }
    for (int i = 0; i < c.n_shapes; ++i) {
        const auto& si = s->shapes[i];
        long long te = t;
        if (si.tstop >= 0) te = t < si.tstop ? t : (t < si.tstop + 100 ? si.tstop : t - 100);
        Shape& o = F.shapes[i];
        o.w = si.w;
        o.h = si.h;
        o.ellipse = si.ellipse;
        o.col = si.col;
        o.x = reflect_pos(si.x0 + si.vx * te, (long long)(c.width - si.w) * 256);
        o.y = reflect_pos(si.y0 + si.vy * te, (long long)(c.height - si.h) * 256);
    }
    return F;
}

}  // namespace

extern "C" {

lvbgs_status lvsynth_preset(int config, int index, uint64_t base, lvsynth_config* o) {
    if (!o) return LVBGS_BAD_ARG;
    std::memset(o, 0, sizeof(*o));
    if (config == 0) {
        *o = lvsynth_config{320, 240, 3, base, 3000, 3, 20, 60, 256, 768, 0, 0, 0, 0, 200};
    } else if (config == 1) {
        *o = lvsynth_config{1920, 1080, 3, base, 4000, 8, 40, 200, 128, 1024, 1, 1, 1, 2, 500};
    } else if (config == 3) {
        if (index < 0 || index >= 64) return LVBGS_BAD_ARG;
        int W, H;
        if (index < 16) W = 320, H = 240;
        else if (index < 40) W = 640, H = 480;
        else if (index < 56) W = 1280, H = 720;
        else W = 1920, H = 1080;
        const uint64_t seed = base * 1000003ull + (uint64_t)index;
        const int C = (index % 4 == 3) ? 1 : 3;
        const int sigma = rnd_range(seed, 1, 0, 2000, 6000);
        const int ns = rnd_range(seed, 2, 0, 2, 10);
        *o = lvsynth_config{W, H, C, seed, sigma, ns, 20, 60, 256, 768, 0, 0, 0, 0, 300};
    } else if (config == 2) {
        // thermal-like 640x480 gray: six warm blobs (radius 10-40), random walks of 1-5 px per frame
        if (index != 0) return LVBGS_BAD_ARG;
        *o = lvsynth_config{640, 480, 1, base * 1000003ull + 2u, 2000, 6, 10, 40, 1, 5, 1, 0, 0, 0, 300, 1};
    } else if (config == 4) {
        // serving streams: index = 2 * resolution class (320x240, 640x480, 1280x720, 1920x1080)
        // + (1 for single-channel); content as in the 64-stream mix, one sequence per base seed
        if (index < 0 || index >= 8) return LVBGS_BAD_ARG;
        static const int kW[4] = {320, 640, 1280, 1920}, kH[4] = {240, 480, 720, 1080};
        const int W = kW[index / 2], H = kH[index / 2], C = (index & 1) ? 1 : 3;
        const uint64_t seed = base * 1000003ull + 64u + (uint64_t)index;
        const int sigma = rnd_range(seed, 1, 0, 2000, 6000);
        const int ns = rnd_range(seed, 2, 0, 2, 10);
        *o = lvsynth_config{W, H, C, seed, sigma, ns, 20, 60, 256, 768, 0, 0, 0, 0, 1800};
    } else {
        return LVBGS_UNSUPPORTED;
    }
    return LVBGS_OK;
}

lvbgs_status lvsynth_create(const lvsynth_config* cfg, lvsynth_handle* out) {
    if (!cfg || !out) return LVBGS_BAD_ARG;
    *out = nullptr;
    if (cfg->width < 8 || cfg->height < 8 || (cfg->channels != 1 && cfg->channels != 3) || cfg->n_shapes < 0 ||
        cfg->n_shapes > LVSYNTH_MAX_SHAPES || cfg->shape_min < 1 || cfg->shape_max < cfg->shape_min ||
        cfg->noise_sigma_milli < 0)
        return LVBGS_BAD_ARG;
    lvsynth_scene* s = new lvsynth_scene();
    s->cfg = *cfg;
    if (cfg->thermal) {
        if (cfg->speed_min_q8 < 0 || cfg->speed_max_q8 < cfg->speed_min_q8) {
            delete s;
            return LVBGS_BAD_ARG;
        }
        build_thermal_texture(s);
    } else {
        build_texture(s);
    }
    // falloff exp(-2 u) (sigma = radius/2) in 1/256 over u = d^2/r^2 in [0, 4)
    for (int i = 0; i < kFalloffN; ++i) s->falloff[i] = (uint16_t)std::lround(256.0 * std::exp(-2.0 * i / 256.0));
    for (int i = 0; i < kRipplePeriod; ++i) s->ripple[i] = (int8_t)std::lround(20.0 * std::sin(2.0 * M_PI * i / kRipplePeriod));
    const uint64_t seed = cfg->seed;
    s->rx0 = cfg->width > kRippleW ? rnd_range(seed, 10, 0, 0, cfg->width - kRippleW) : 0;
    s->ry0 = cfg->height > kRippleH ? rnd_range(seed, 11, 0, 0, cfg->height - kRippleH) : 0;
    const int smax = std::min(cfg->shape_max, std::min(cfg->width, cfg->height) - 1);
    const int smin = std::min(cfg->shape_min, smax);
    for (int i = 0; i < cfg->n_shapes; ++i) {
        auto& sh = s->shapes[i];
        const uint32_t a = 100 + i;
        sh.w = rnd_range(seed, a, 1, smin, smax);
        sh.h = rnd_range(seed, a, 2, smin, smax);
        sh.ellipse = cfg->ellipses_only ? 1 : (int)(rnd32(seed, a, 3, 0, 0) & 1u);
        sh.col = rnd32(seed, a, 4, 0, 1) & 0xffffffu;
        sh.x0 = (long long)rnd_range(seed, a, 5, 0, cfg->width - sh.w) * 256;
        sh.y0 = (long long)rnd_range(seed, a, 6, 0, cfg->height - sh.h) * 256;
        const int vx = rnd_range(seed, a, 7, cfg->speed_min_q8, cfg->speed_max_q8);
        const int vy = rnd_range(seed, a, 8, cfg->speed_min_q8, cfg->speed_max_q8);
        sh.vx = (rnd32(seed, a, 9, 0, 2) & 1u) ? vx : -vx;
        sh.vy = (rnd32(seed, a, 9, 0, 3) & 1u) ? vy : -vy;
        sh.tstop = i < cfg->n_stopping ? 50 + 150 * i : -1;
        if (cfg->thermal) {
            // blob: w = radius, col = intensity 180..240, (x0, y0) = centre in whole pixels
            const int r = rnd_range(seed, a, 1, cfg->shape_min, cfg->shape_max);
            sh.w = sh.h = r;
            sh.col = (uint32_t)rnd_range(seed, a, 4, 180, 240);
            sh.x0 = rnd_range(seed, a, 5, std::min(r, cfg->width - 1), std::max(r, cfg->width - 1 - r));
            sh.y0 = rnd_range(seed, a, 6, std::min(r, cfg->height - 1), std::max(r, cfg->height - 1 - r));
        }
    }
    *out = s;
    return LVBGS_OK;
}

void lvsynth_destroy(lvsynth_handle h) {
    if (!h) return;
    cudaFree(h->d_tex);
    cudaFree(h->d_ripple);
    cudaFree(h->d_falloff);
    delete h;
}

lvbgs_status lvsynth_render(lvsynth_handle h, int t, uint8_t* frame, uint8_t* gt) {
    if (!h || t < 0) return LVBGS_BAD_ARG;
    const FrameParams F = frame_params(h, t);
    std::vector<uint8_t> scratch;
    uint8_t* out = frame;
    if (!out) {
        scratch.resize((size_t)F.W * F.H * F.C);
        out = scratch.data();
    }
    for (int y = 0; y < F.H; ++y)
        for (int x = 0; x < F.W; ++x) render_px(F, h->tex.data(), h->ripple, h->falloff, x, y, out, gt);
    return LVBGS_OK;
}

lvbgs_status lvsynth_render_device(lvsynth_handle h, int t, uint8_t* frame, uint8_t* gt, void* stream) {
    if (!h || t < 0 || !frame) return LVBGS_BAD_ARG;
    if (!h->d_tex) {
        if (cudaMalloc(&h->d_tex, h->tex.size()) != cudaSuccess) return LVBGS_OOM;
        if (cudaMalloc(&h->d_ripple, sizeof(h->ripple)) != cudaSuccess) return LVBGS_OOM;
        if (cudaMemcpy(h->d_tex, h->tex.data(), h->tex.size(), cudaMemcpyHostToDevice) != cudaSuccess) return LVBGS_DEVICE_ERROR;
        if (cudaMemcpy(h->d_ripple, h->ripple, sizeof(h->ripple), cudaMemcpyHostToDevice) != cudaSuccess)
            return LVBGS_DEVICE_ERROR;
        if (cudaMalloc(&h->d_falloff, sizeof(h->falloff)) != cudaSuccess) return LVBGS_OOM;
        if (cudaMemcpy(h->d_falloff, h->falloff, sizeof(h->falloff), cudaMemcpyHostToDevice) != cudaSuccess)
            return LVBGS_DEVICE_ERROR;
    }
    const FrameParams F = frame_params(h, t);
    render_kernel<<<512, 256, 0, (cudaStream_t)stream>>>(F, h->d_tex, h->d_ripple, h->d_falloff, frame, gt);
    return cudaGetLastError() == cudaSuccess ? LVBGS_OK : LVBGS_DEVICE_ERROR;
}

}  // extern "C"
