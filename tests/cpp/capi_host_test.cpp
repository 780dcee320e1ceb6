// C++ host-side use of the imaging C ABI, as a C++ caller (the reference's own language) drives
// it: an imager handle on device and host buffers, deterministic repeatability, the free
// functions in the reference's call order, and the serving runtime.  Builds with g++ against
// include/blink_imager_gb300.h and the library; exits non-zero on the first failed check.
#include <blink_imager_gb300.h>
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

namespace {

int failures = 0;

#define CHECK(cond, ...)                                \
    do {                                                \
        if (!(cond)) {                                  \
            std::fprintf(stderr, "FAILED %s:%d: ", __FILE__, __LINE__); \
            std::fprintf(stderr, __VA_ARGS__);          \
            std::fprintf(stderr, "\n");                \
            ++failures;                                 \
        }                                               \
    } while (0)

void ok(int status, const char *what) {
    if (status != BGI_OK) {
        std::fprintf(stderr, "%s: status %d: %s\n", what, status, bgi_last_error());
        std::exit(2);
    }
}

double rel_l2(const std::vector<float> &a, const std::vector<float> &b) {
    double num = 0, den = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        num += (double)(a[i] - b[i]) * (a[i] - b[i]);
        den += (double)b[i] * b[i];
    }
    return std::sqrt(num / (den > 0 ? den : 1));
}

}  // namespace

int main() {
    const int n_ant = 48, T = 2, C = 3, N = 128;
    const int B = n_ant * (n_ant + 1) / 2, n_images = T * C;
    std::mt19937 rng(7);
    std::uniform_real_distribution<double> pos(-35.0, 35.0);
    std::normal_distribution<float> gauss(0.f, 1.f);
    // zenith UVW of the lower-triangular baselines (u = -(x_i - x_j), src/antenna_positions.cpp:81-89)
    std::vector<double> x(n_ant), y(n_ant), cable(n_ant);
    for (int a = 0; a < n_ant; ++a) x[a] = pos(rng), y[a] = pos(rng), cable[a] = 100.0 + pos(rng);
    std::vector<float> u(B), v(B), w(B, 0.f);
    std::vector<int> flags(B, 0);
    for (int i = 0, b = 0; i < n_ant; ++i)
        for (int j = 0; j <= i; ++j, ++b) {
            u[b] = (float)(-(x[i] - x[j]));
            v[b] = (float)(-(y[i] - y[j]));
            flags[b] = i == j;  // autos flagged
        }
    std::vector<double> freqs(C);
    for (int c = 0; c < C; ++c) freqs[c] = 150e6 + 1.28e6 * c;
    std::vector<std::complex<float>> vis((size_t)n_images * B * 4);
    for (auto &z : vis) z = {gauss(rng), gauss(rng)};

    // ---- imager handle: device buffers, then host buffers --------------------------------
    bgi_config cfg{};
    cfg.n_pixels = N;
    cfg.oversampling_factor = 2.0f;
    cfg.pol = BGI_POL_XX;
    cfg.min_uv = -1000.0;
    cfg.device = 0;
    bgi_imager *im = nullptr;
    ok(bgi_create(&cfg, &im), "create");
    ok(bgi_set_array(im, n_ant, 1, u.data(), v.data(), w.data(), flags.data(), cable.data()), "set_array");
    ok(bgi_set_frequencies(im, C, freqs.data()), "set_frequencies");
    const size_t img_floats = (size_t)n_images * N * N * 2;
    float *d_vis = nullptr, *d_img = nullptr;
    ok(cudaMalloc(&d_vis, sizeof(std::complex<float>) * vis.size()) == cudaSuccess ? BGI_OK : BGI_ERR_CUDA, "malloc");
    ok(cudaMalloc(&d_img, sizeof(float) * img_floats) == cudaSuccess ? BGI_OK : BGI_ERR_CUDA, "malloc");
    cudaMemcpy(d_vis, vis.data(), sizeof(std::complex<float>) * vis.size(), cudaMemcpyHostToDevice);
    ok(bgi_set_deterministic(im, 1), "deterministic");
    const unsigned flags_corr = BGI_APPLY_GEOMETRIC | BGI_APPLY_CABLE;
    ok(bgi_image(im, d_vis, T, flags_corr, d_img, nullptr), "image");
    std::vector<float> a(img_floats), b(img_floats), hosted(img_floats);
    cudaMemcpy(a.data(), d_img, sizeof(float) * img_floats, cudaMemcpyDeviceToHost);
    ok(bgi_image(im, d_vis, T, flags_corr, d_img, nullptr), "image again");
    cudaMemcpy(b.data(), d_img, sizeof(float) * img_floats, cudaMemcpyDeviceToHost);
    CHECK(std::memcmp(a.data(), b.data(), sizeof(float) * img_floats) == 0, "deterministic images differ");
    ok(bgi_image_host(im, reinterpret_cast<const float *>(vis.data()), T, flags_corr, hosted.data(), nullptr),
       "image_host");
    CHECK(std::memcmp(a.data(), hosted.data(), sizeof(float) * img_floats) == 0, "host images differ");
    std::vector<uint32_t> sums(n_images);
    ok(bgi_last_weight_sums(im, sums.data(), n_images, nullptr), "weight sums");
    for (int i = 0; i < n_images; ++i) CHECK(sums[i] > 0 && sums[i] % 2 == 0, "weight sum %u", sums[i]);

    // ---- the reference's call order through the free functions, on corrected visibilities --
    double du = 0, dv = 0, umax = 0, vmax = 0;
    ok(bgi_get_uv_cell(im, &du, &dv, &umax, &vmax), "uv cell");
    float *d_grid = nullptr, *d_cnt = nullptr, *d_w = nullptr, *d_u = nullptr, *d_v = nullptr, *d_fn = nullptr,
          *d_img2 = nullptr;
    int *d_flags = nullptr;
    double *d_freqs = nullptr, *d_cable = nullptr;
    cudaMalloc(&d_grid, sizeof(float) * img_floats);
    cudaMalloc(&d_img2, sizeof(float) * img_floats);
    cudaMalloc(&d_cnt, sizeof(float) * (size_t)C * N * N);
    cudaMalloc(&d_fn, sizeof(float) * C);
    cudaMalloc(&d_u, sizeof(float) * B);
    cudaMalloc(&d_v, sizeof(float) * B);
    cudaMalloc(&d_w, sizeof(float) * B);
    cudaMalloc(&d_flags, sizeof(int) * B);
    cudaMalloc(&d_freqs, sizeof(double) * C);
    cudaMalloc(&d_cable, sizeof(double) * n_ant);
    cudaMemcpy(d_u, u.data(), sizeof(float) * B, cudaMemcpyHostToDevice);
    cudaMemcpy(d_v, v.data(), sizeof(float) * B, cudaMemcpyHostToDevice);
    cudaMemcpy(d_w, w.data(), sizeof(float) * B, cudaMemcpyHostToDevice);
    cudaMemcpy(d_flags, flags.data(), sizeof(int) * B, cudaMemcpyHostToDevice);
    cudaMemcpy(d_freqs, freqs.data(), sizeof(double) * C, cudaMemcpyHostToDevice);
    cudaMemcpy(d_cable, cable.data(), sizeof(double) * n_ant, cudaMemcpyHostToDevice);
    ok(bgi_apply_geometric_corrections_gpu(d_vis, n_ant, C, T, d_w, 1, d_freqs, nullptr), "geometric");
    ok(bgi_apply_cable_lengths_corrections_gpu(d_vis, n_ant, C, T, d_cable, d_freqs, nullptr), "cable");
    cudaMemset(d_grid, 0, sizeof(float) * img_floats);
    cudaMemset(d_cnt, 0, sizeof(float) * (size_t)C * N * N);
    ok(bgi_gridding_gpu(d_vis, n_ant, C, T, d_u, d_v, 1, d_flags, nullptr, d_freqs, du, dv, N, -1000.0, BGI_POL_XX,
                        BGI_COUNTERS_FIRST_INTERVAL, d_cnt, d_grid, nullptr),
       "gridding");
    ok(bgi_fft_inverse_gpu(d_grid, d_img2, N, n_images, nullptr), "fft");
    ok(bgi_vector_sum_gpu(d_cnt, (int64_t)N * N, C, d_fn, nullptr), "vector sum");
    ok(bgi_fft_shift_and_norm_gpu(d_img2, N, N, n_images, d_fn, C, nullptr), "shift and norm");
    std::vector<float> plain(img_floats);
    cudaMemcpy(plain.data(), d_img2, sizeof(float) * img_floats, cudaMemcpyDeviceToHost);
    // interval 0: the per-channel norm equals the per-image one, so the images agree
    const size_t per_interval = (size_t)C * N * N * 2;
    std::vector<float> p0(plain.begin(), plain.begin() + per_interval), a0(a.begin(), a.begin() + per_interval);
    CHECK(rel_l2(p0, a0) < 1e-5, "free-function images differ from the handle's: %g", rel_l2(p0, a0));

    // ---- serving runtime ------------------------------------------------------------------
    bgi_server_config sc{};
    sc.device = 0;
    sc.max_slots = 2;
    sc.reserve_bytes = 256u << 20;
    sc.deterministic = 1;
    bgi_server *sv = nullptr;
    ok(bgi_server_create(&sc, &sv), "server create");
    int aid = -1;
    ok(bgi_server_add_array(sv, &cfg, n_ant, 1, u.data(), v.data(), w.data(), flags.data(), cable.data(), C,
                            freqs.data(), &aid),
       "server add_array");
    std::vector<float> served(img_floats), served2(img_floats);
    uint64_t t1 = 0, t2 = 0;
    ok(bgi_server_submit(sv, aid, BGI_VIS_C64, vis.data(), nullptr, T, flags_corr, served.data(), &t1), "submit");
    ok(bgi_server_submit(sv, aid, BGI_VIS_C64, vis.data(), nullptr, T, flags_corr, served2.data(), &t2), "submit");
    int st1 = -99, st2 = -99;
    ok(bgi_server_wait(sv, t1, -1, &st1), "wait");
    ok(bgi_server_wait(sv, t2, -1, &st2), "wait");
    CHECK(st1 == BGI_OK && st2 == BGI_OK, "request status %d %d", st1, st2);
    CHECK(std::memcmp(a.data(), served.data(), sizeof(float) * img_floats) == 0, "served images differ");
    CHECK(std::memcmp(a.data(), served2.data(), sizeof(float) * img_floats) == 0, "served images differ");
    bgi_server_stats stats{};
    ok(bgi_server_get_stats(sv, &stats), "stats");
    CHECK(stats.completed == 2 && stats.p50_ms > 0, "server stats");
    ok(bgi_server_destroy(sv), "server destroy");

    ok(bgi_destroy(im), "destroy");
    for (void *p : {(void *)d_vis, (void *)d_img, (void *)d_grid, (void *)d_img2, (void *)d_cnt, (void *)d_fn,
                    (void *)d_u, (void *)d_v, (void *)d_w, (void *)d_flags, (void *)d_freqs, (void *)d_cable})
        cudaFree(p);
    if (failures) return 1;
    std::printf("C++ host checks passed\n");
    return 0;
}
