// capi_driver.cpp -- a C++ host program driving the step through the C-ABI,
// the way CERNsource/time_integration.f:175-183 drives single_step from its
// time loop (and sph.f:341-348 calls time_integration).
//
//   capi_driver <state.bin> <out.bin> <steps> <refresh>
//
// state.bin: int32 dim, int64 n_fluid, int64 n_wall, float32 dt, then the
// armando_params record (sizeof(armando_params) bytes, the header's layout),
// then the arrays x[n*dim], v[n*dim], mass[n], rho[n], p[n], u[n], h[n],
// itype[n] (int32), dvdt[n*dim], dudt[n]. The program runs `steps` leapfrog
// iterations as time_integration does: one armando_integrate call per block of
// `refresh` iterations (the caller's arrays are the state between blocks), and
// writes the arrays back in the same layout (without the header).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "armando.h"

namespace {

template <class T>
bool read_into(FILE* f, std::vector<T>& v, size_t n) {
    v.resize(n);
    return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

template <class T>
bool write_from(FILE* f, const std::vector<T>& v) {
    return v.empty() || std::fwrite(v.data(), sizeof(T), v.size(), f) == v.size();
}

int die(const char* what, armando_ctx* ctx) {
    std::fprintf(stderr, "capi_driver: %s: %s\n", what, armando_last_error(ctx));
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: capi_driver <state.bin> <out.bin> <steps> <refresh>\n");
        return 1;
    }
    const int steps = std::atoi(argv[3]), refresh = std::atoi(argv[4]);
    if (steps < 0 || refresh < 1) return 1;
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 1;
    int32_t dim = 0;
    int64_t nf = 0, nw = 0;
    float dt = 0.f;
    armando_params prm;
    if (std::fread(&dim, 4, 1, in) != 1 || std::fread(&nf, 8, 1, in) != 1 ||
        std::fread(&nw, 8, 1, in) != 1 || std::fread(&dt, 4, 1, in) != 1 ||
        std::fread(&prm, sizeof prm, 1, in) != 1)
        return 1;
    const size_t n = (size_t)(nf + nw), nd = n * (size_t)dim;
    std::vector<float> x, v, m, rho, p, u, h, dvdt, dudt;
    std::vector<int32_t> itype;
    bool ok = read_into(in, x, nd) && read_into(in, v, nd) && read_into(in, m, n) &&
              read_into(in, rho, n) && read_into(in, p, n) && read_into(in, u, n) &&
              read_into(in, h, n) && read_into(in, itype, n) && read_into(in, dvdt, nd) &&
              read_into(in, dudt, n);
    std::fclose(in);
    if (!ok) return 1;

    if (armando_abi_version() != ARMANDO_ABI_VERSION) return die("ABI version", nullptr);
    armando_ctx* ctx = nullptr;
    if (armando_create(&ctx, &prm, dim, nf, nw, ARMANDO_MEM_HOST) != ARMANDO_OK)
        return die("armando_create", nullptr);
    // do its = 1, steps (time_integration.f:131): neighbour refresh every
    // `refresh` iterations is one call per block here.
    for (int its = 1; its <= steps; its += refresh) {
        const int k = (steps - its + 1 < refresh) ? steps - its + 1 : refresh;
        if (armando_integrate(ctx, x.data(), v.data(), m.data(), rho.data(), p.data(), u.data(),
                              h.data(), itype.data(), dvdt.data(), dudt.data(), dt, its, k) !=
            ARMANDO_OK)
            return die("armando_integrate", ctx);
    }
    armando_stats st;
    if (armando_get_stats(ctx, &st) != ARMANDO_OK) return die("armando_get_stats", ctx);
    std::printf("steps_done %lld gpu_launches %lld\n", (long long)st.steps_done,
                (long long)st.gpu_launches);
    if (armando_destroy(ctx) != ARMANDO_OK) return die("armando_destroy", nullptr);

    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 1;
    ok = write_from(out, x) && write_from(out, v) && write_from(out, m) && write_from(out, rho) &&
         write_from(out, p) && write_from(out, u) && write_from(out, h) && write_from(out, itype) &&
         write_from(out, dvdt) && write_from(out, dudt);
    std::fclose(out);
    return ok ? 0 : 1;
}
