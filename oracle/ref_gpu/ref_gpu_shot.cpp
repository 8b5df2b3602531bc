/*
 * The reference's own CUDA kernels on the GPU, one shot sequenced as
 * src/main.c:318-495 sequences it (test and benchmark infrastructure only:
 * built into oracle/_ref/ beside the reference's kernels, which
 * `make -C oracle ref-gpu` compiles unchanged for sm_103a from the
 * reference checkout into oracle/_ref/parallelcalls.cubin; nothing in the
 * product links or loads either).
 *
 * The launch grids and streams are src/serialcalls.cu's: 32 x 32 blocks over
 * the grid (512-thread 1-D blocks for the CPML profiles); per forward step the
 * snapshot of the previous level goes to pinned host memory on stream1 while
 * SecondDerivate_P, PSI_F and ZETA_F run on stream2 and propagator_F on the
 * legacy default stream; per adjoint step the snapshot comes back on stream1,
 * entryPoint .. retroPropagation run on stream2 and GRADIENT on the legacy
 * stream.  Buffers are allocated and aliased as src/main.c:140-228 does
 * (F = P + nx nz in one allocation per level; the adjoint's zeta and psi
 * arrays alias the forward's).
 *
 *   ref_gpu_shot <cubin> <dir> nx nz nt cpml dh dt f sx sz shots
 *
 * <dir> holds vel.f32, eps.f32, delta.f32 (the model, [nz][nx]) and obs.f32
 * (the observed record of the shot, [nt][nx] as src/main.c keeps shot1).
 * sx, sz are the reference's 1-based source coordinates.  The shot is run
 * `shots` times; the program prints one line of JSON (seconds per shot of
 * each run, the misfit) and writes gcx.f32, gcz.f32, gdx.f32 and res.f32 of
 * the last run to <dir>.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define CK(x)                                                                                 \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) {                                                              \
            fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            exit(2);                                                                          \
        }                                                                                     \
    } while (0)

static std::vector<float> read_f32(const std::string &path, size_t n)
{
    std::vector<float> v(n);
    FILE *f = fopen(path.c_str(), "rb");
    if (!f || fread(v.data(), sizeof(float), n, f) != n) {
        fprintf(stderr, "cannot read %zu floats from %s\n", n, path.c_str());
        exit(2);
    }
    fclose(f);
    return v;
}

static void write_f32(const std::string &path, const float *d, size_t n)
{
    std::vector<float> h(n);
    CK(cudaMemcpy(h.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost));
    FILE *f = fopen(path.c_str(), "wb");
    if (!f || fwrite(h.data(), sizeof(float), n, f) != n) exit(2);
    fclose(f);
}

struct Lib {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t get(const char *name)
    {
        cudaKernel_t k = nullptr;
        CK(cudaLibraryGetKernel(&k, lib, name));
        return k;
    }
};

// One launch: the argument list as the kernel's prototype (include/parallelcalls.h) orders it.
template <typename... A> static void launch(cudaKernel_t k, dim3 g, dim3 b, cudaStream_t s, A... a)
{
    void *args[] = {(void *)&a...};
    CK(cudaLaunchKernel((const void *)k, g, b, args, 0, s));
}

int main(int argc, char **argv)
{
    if (argc != 13) {
        fprintf(stderr, "usage: %s cubin dir nx nz nt cpml dh dt f sx sz shots\n", argv[0]);
        return 1;
    }
    const std::string dir = argv[2];
    const int nx = atoi(argv[3]), nz = atoi(argv[4]), nt = atoi(argv[5]), CPML = atoi(argv[6]);
    const float dh = (float)atof(argv[7]), dt = (float)atof(argv[8]), f = (float)atof(argv[9]);
    const int sx = atoi(argv[10]), sz = atoi(argv[11]), nrun = atoi(argv[12]);
    const size_t n = (size_t)nx * nz;

    Lib L;
    CK(cudaLibraryLoadFromFile(&L.lib, argv[1], nullptr, nullptr, 0, nullptr, nullptr, 0));
    cudaKernel_t k_pre = L.get("pre_variables"), k_cx = L.get("CPML_x"), k_cz = L.get("CPML_z");
    cudaKernel_t k_psif = L.get("PSI_F"), k_zetaf = L.get("ZETA_F"), k_prop = L.get("propagator_F");
    cudaKernel_t k_res = L.get("res"), k_d2p = L.get("SecondDerivate_P"), k_retro = L.get("retroPropagation");
    cudaKernel_t k_entry = L.get("entryPoint"), k_psir = L.get("PSI_R"), k_d2 = L.get("secondDerivate");
    cudaKernel_t k_zetar = L.get("ZETA_R"), k_grad = L.get("GRADIENT");

    // constants as src/main.c:48-55 forms them (float arithmetic)
    const float R = 1e-6f, Lw = CPML * dh, d0 = -3 * logf(R) / (2 * Lw), Vmax = 6000;
    const float dh2 = dh * dh, C = (dt * dt) / dh2;

    auto dalloc = [](size_t count) {
        float *p = nullptr;
        CK(cudaMalloc(&p, count * sizeof(float)));
        CK(cudaMemset(p, 0, count * sizeof(float)));
        return p;
    };
    float *vel = dalloc(n), *eps = dalloc(n), *del = dalloc(n), *v_hor = dalloc(n), *v_po = dalloc(n),
          *v_nmo = dalloc(n);
    float *a_x = dalloc(nx), *b_x = dalloc(nx), *a_z = dalloc(nz), *b_z = dalloc(nz), *source = dalloc(nt);
    float *psi_px = dalloc(n), *psi_fz = dalloc(n), *z_px = dalloc(n), *z_fz = dalloc(n), *aten_p = dalloc(n),
          *aten_f = dalloc(n);
    float *P_pre = dalloc(2 * n), *P_past = dalloc(2 * n), *P_pre2 = dalloc(2 * n);
    float *PF = dalloc(n), *shot1 = dalloc((size_t)nx * nt), *shot2 = dalloc((size_t)nx * nt),
          *Res = dalloc((size_t)nx * nt);
    float *aux1 = dalloc(n), *aux2 = dalloc(n), *aux3 = dalloc(n), *aux4 = dalloc(n);
    float *atenxcx = dalloc(n), *atenxcz = dalloc(n), *atenzdx = dalloc(n), *atenzcz = dalloc(n);
    float *zitaxcx = z_px, *zitaxcz = z_fz, *zitazdx = aten_f, *zitazcz = aten_p;  // src/main.c:184-187
    float *psixcx = dalloc(n), *psixcz = dalloc(n), *psizdx = psi_px, *psizcz = psi_fz;
    float *p2cx = dalloc(n), *p2cz = dalloc(n), *r2dx = dalloc(n), *r2cz = dalloc(n);
    float *gcx = dalloc(n), *gcz = dalloc(n), *gdx = dalloc(n), *p2 = dalloc(n), *r2 = dalloc(n);
    float *PF_h = nullptr;
    CK(cudaMallocHost(&PF_h, (size_t)nt * 2 * n * sizeof(float)));
    std::vector<float> res_h((size_t)nx * nt);

    {
        std::vector<float> a = read_f32(dir + "/vel.f32", n), b = read_f32(dir + "/eps.f32", n),
                           c = read_f32(dir + "/delta.f32", n), o = read_f32(dir + "/obs.f32", (size_t)nx * nt);
        CK(cudaMemcpy(vel, a.data(), n * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(eps, b.data(), n * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(del, c.data(), n * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(shot1, o.data(), (size_t)nx * nt * 4, cudaMemcpyHostToDevice));
        // Ricker wavelet, src/main.c:328-333 (float time accumulated on the host)
        std::vector<float> s(nt);
        float t = 0;
        for (int it = 0; it < nt; it++) {
            t += dt;
            s[it] = (float)(1 * (1 - 2 * pow(M_PI * f * (t - (1 / f)), 2)) * exp(-pow(M_PI * f * (t - (1 / f)), 2)));
        }
        CK(cudaMemcpy(source, s.data(), nt * 4, cudaMemcpyHostToDevice));
    }
    const dim3 grid((unsigned)ceil(nx / 32.0f), (unsigned)ceil(nz / 32.0f)), block(32, 32);
    launch(k_pre, grid, block, 0, vel, eps, del, v_hor, v_po, v_nmo, nx, nz);
    launch(k_cx, dim3((unsigned)ceil(nx / 512.0f)), dim3(512), 0, a_x, b_x, CPML, Vmax, nx, dt, dh, f, d0, Lw);
    launch(k_cz, dim3((unsigned)ceil(nz / 512.0f)), dim3(512), 0, a_z, b_z, CPML, Vmax, nz, dt, dh, f, d0, Lw);
    CK(cudaDeviceSynchronize());

    cudaStream_t stream1, stream2;
    CK(cudaStreamCreate(&stream1));
    CK(cudaStreamCreate(&stream2));
    std::vector<double> secs;
    float fi = 0;
    for (int run = 0; run < nrun; run++) {
        CK(cudaDeviceSynchronize());
        const auto t0 = std::chrono::steady_clock::now();
        for (float *p : {gcx, gcz, gdx}) CK(cudaMemset(p, 0, n * 4));
        for (float *p : {psi_px, psi_fz, aten_p, aten_f, z_px, z_fz}) CK(cudaMemset(p, 0, n * 4));
        CK(cudaMemset(P_pre, 0, 2 * n * 4));
        CK(cudaMemset(P_past, 0, 2 * n * 4));
        float *Pp = P_past, *Pc = P_pre;  // src/main.c swaps the two levels after each step
        for (int it = 0; it < nt; it++) {
            float *Fp = Pp + n, *Fc = Pc + n;
            CK(cudaMemcpyAsync(&PF_h[2 * (size_t)it * n], Pp, 2 * n * 4, cudaMemcpyDeviceToHost, stream1));
            launch(k_d2p, grid, block, stream2, Pc, Fc, p2, r2, dh2, nx, nz);
            launch(k_psif, grid, block, stream2, Pc, Fc, a_x, b_x, a_z, b_z, psi_px, psi_fz, nx, nz, dh, CPML);
            launch(k_zetaf, grid, block, stream2, p2, r2, Pc, Fc, a_x, b_x, a_z, b_z, psi_px, psi_fz, z_px, z_fz,
                   aten_p, aten_f, nx, nz, dh, dh2, CPML);
            launch(k_prop, grid, block, 0, p2, r2, PF, Pc, Fc, Pp, Fp, v_hor, v_po, v_nmo, aten_p, aten_f, source,
                   shot2, C, dh2, nx, nz, sx, sz, it, CPML);
            std::swap(Pp, Pc);
        }
        launch(k_res, dim3((unsigned)ceil(nx / 32.0f), (unsigned)ceil(nt / 32.0f)), block, 0, Res, shot1, shot2, nx,
               nt);
        CK(cudaMemcpy(res_h.data(), Res, (size_t)nx * nt * 4, cudaMemcpyDeviceToHost));
        fi = 0;
        for (size_t j = 0; j < (size_t)nx * nt; j++) fi += powf(res_h[j], 2);
        fi = fi / 2;
        CK(cudaMemset(P_pre, 0, 2 * n * 4));
        CK(cudaMemset(P_past, 0, 2 * n * 4));
        for (float *p : {psixcz, psixcx, psizcz, psizdx, atenxcx, atenxcz, atenzdx, atenzcz, zitaxcx, zitaxcz,
                         zitazdx, zitazcz})
            CK(cudaMemset(p, 0, n * 4));
        Pp = P_past;
        Pc = P_pre;
        for (int it = 0; it < nt; it++) {
            float *Fp = Pp + n, *Fc = Pc + n;
            CK(cudaMemcpyAsync(P_pre2, &PF_h[(size_t)(nt - it - 1) * n * 2], 2 * n * 4, cudaMemcpyHostToDevice,
                               stream1));
            launch(k_entry, grid, block, stream2, Pc, Fc, aux1, aux2, aux3, aux4, v_hor, v_po, v_nmo, nx, nz);
            launch(k_d2, grid, block, stream2, aux1, aux2, aux3, aux4, p2cx, p2cz, r2dx, r2cz, dh2, nx, nz);
            launch(k_psir, grid, block, stream2, aux1, aux2, aux3, aux4, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx,
                   psizcz, nx, nz, dh, CPML);
            launch(k_zetar, grid, block, stream2, p2cx, p2cz, r2dx, r2cz, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx,
                   psizcz, zitaxcx, zitaxcz, zitazdx, zitazcz, atenxcx, atenxcz, atenzdx, atenzcz, nx, nz, dh, dh2,
                   CPML);
            launch(k_retro, grid, block, stream2, PF, Pc, Fc, Pp, Fp, Res, C, dh2, nx, nz, nt, sz, it, CPML, p2cx,
                   p2cz, r2dx, r2cz, atenxcx, atenxcz, atenzdx, atenzcz);
            launch(k_grad, grid, block, 0, P_pre2, P_pre2 + n, Pp, Fp, gcx, gcz, gdx, dh2, dt, nx, nz);
            std::swap(Pp, Pc);
        }
        CK(cudaDeviceSynchronize());
        secs.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
    CK(cudaGetLastError());
    write_f32(dir + "/gcx.f32", gcx, n);
    write_f32(dir + "/gcz.f32", gcz, n);
    write_f32(dir + "/gdx.f32", gdx, n);
    write_f32(dir + "/res.f32", Res, (size_t)nx * nt);
    printf("{\"seconds_per_shot\": [");
    for (size_t k = 0; k < secs.size(); k++) printf("%s%.6f", k ? ", " : "", secs[k]);
    printf("], \"misfit\": %.9g}\n", (double)fi);
    CK(cudaFreeHost(PF_h));
    return 0;
}
