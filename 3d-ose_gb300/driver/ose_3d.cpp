// ose_3d - host driver over libose3d.so that reproduces the reference
// program's flow and files (ose_3d.cu:70-304):
//   ./output/qshot2.bin    receiver gather of the last shot, [ig][it] float32
//   ./output/partest.txt   parameter dump (output_par layout)
//   ./temp/ricker_card.bin, ./temp/hilbert_card.bin   the shot's source traces
//   ./temp/att_x_0.bin     x sponge profile, 300 floats (zero-padded) as written
//                          by Alloc_mulGPU
//   ./wf/{p,q}-<it>-single.bin (only with wf_every=K): padded P / Q every K
//                          steps in the [y][x][z] dump layout
// Parameters default to the reference's hard-coded values and are overridden
// by key=value arguments with the same names (nx=..., boundary=..., nt=...,
// fm=..., model=path, wf_every=K, nsteps=K).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include <string>
#include <vector>

#include "ose3d.h"

namespace {

bool set_param(ose_params& p, const char* key, const char* val)
{
    struct I { const char* k; int* v; } ints[] = {
        {"nx", &p.nx}, {"ny", &p.ny}, {"nz", &p.nz}, {"bu", &p.bu}, {"bd", &p.bd}, {"bl", &p.bl},
        {"br", &p.br}, {"bf", &p.bf}, {"bb", &p.bb}, {"nt", &p.nt}, {"nshot", &p.nshot},
        {"sxbeg", &p.sxbeg}, {"sybeg", &p.sybeg}, {"szbeg", &p.szbeg}, {"jsx", &p.jsx},
        {"jsy", &p.jsy}, {"jsz", &p.jsz}, {"gxbeg", &p.gxbeg}, {"gybeg", &p.gybeg},
        {"gzbeg", &p.gzbeg}, {"jgx", &p.jgx}, {"jgy", &p.jgy}, {"jgz", &p.jgz},
        {"csdgather", &p.csdgather}, {"sponge_mode", &p.sponge_mode},
        {"hilbert_div_nt", &p.hilbert_div_nt}, {"M", &p.M_override}};
    struct F { const char* k; float* v; } flts[] = {
        {"fm", &p.fm}, {"dt", &p.dt}, {"amp", &p.amp}, {"dx", &p.dx}, {"dy", &p.dy}, {"dz", &p.dz},
        {"cerjan_factor", &p.cerjan_factor}};
    if (!strcmp(key, "boundary")) {
        int b = atoi(val);
        p.bu = p.bd = p.bl = p.br = p.bf = p.bb = b;
        return true;
    }
    for (auto& i : ints)
        if (!strcmp(key, i.k)) { *i.v = atoi(val); return true; }
    for (auto& f : flts)
        if (!strcmp(key, f.k)) { *f.v = (float)atof(val); return true; }
    return false;
}

int write_floats(const char* path, const float* data, size_t n)
{
    FILE* f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "Can not write this file : %s\n", path); return -1; }
    size_t w = fwrite(data, sizeof(float), n, f);
    fclose(f);
    return w == n ? 0 : -1;
}

#define CHECK(call)                                                                  \
    do {                                                                             \
        ose_status s_ = (call);                                                      \
        if (s_ != OSE_OK) {                                                          \
            fprintf(stderr, "%s failed (%d): %s\n", #call, (int)s_, ose_last_error(h)); \
            return 1;                                                                \
        }                                                                            \
    } while (0)

}  // namespace

int main(int argc, char** argv)
{
    ose_params p;
    ose_default_params(&p);
    std::string model = "./input/v3d_nx101_ny101_nz101.bin";
    int wf_every = 0, nsteps = -1;
    for (int i = 1; i < argc; ++i) {
        const char* eq = strchr(argv[i], '=');
        if (!eq) { fprintf(stderr, "argument %s is not key=value\n", argv[i]); return 2; }
        std::string key(argv[i], eq - argv[i]);
        const char* val = eq + 1;
        if (key == "model") model = val;
        else if (key == "wf_every") wf_every = atoi(val);
        else if (key == "nsteps") nsteps = atoi(val);
        else if (!set_param(p, key.c_str(), val)) { fprintf(stderr, "unknown key %s\n", key.c_str()); return 2; }
    }
    if (nsteps < 0 || nsteps > p.nt) nsteps = p.nt;
    mkdir("./output", 0755);
    mkdir("./temp", 0755);
    mkdir("./wf", 0755);

    timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    ose_handle* h = nullptr;
    CHECK(ose_create_from_file(&p, model.c_str(), &h));
    ose_derived d;
    CHECK(ose_get_derived(h, &d));
    printf("nxbnew=%d\tbrnew=%d\n", d.nxb, d.br);
    printf("vmax=%f\nR=%f \ndtR=%f M=%d\n", d.vmax, d.R, d.dtR, d.M);
    {
        std::vector<float> ax(d.nxb > 300 ? d.nxb : 300, 0.f);
        CHECK(ose_get_sponge(h, ax.data(), nullptr, nullptr));
        write_floats("./temp/att_x_0.bin", ax.data(), ax.size());
    }
    const size_t ncell = (size_t)d.nxb * d.nyb * d.nzb;
    std::vector<float> field(wf_every > 0 ? ncell : 0);
    for (int is = 0; is < p.nshot; ++is) {
        CHECK(ose_reset_shot(h, is));
        std::vector<float> ricker(p.nt), hil(p.nt);
        CHECK(ose_get_wavelets(h, ricker.data(), hil.data()));
        write_floats("./temp/ricker_card.bin", ricker.data(), p.nt);
        write_floats("./temp/hilbert_card.bin", hil.data(), p.nt);
        int done = 0;
        while (done < nsteps) {
            int chunk = wf_every > 0 ? wf_every : nsteps - done;
            if (chunk > nsteps - done) chunk = nsteps - done;
            CHECK(ose_run(h, chunk, nullptr));
            done += chunk;
            if (wf_every > 0) {
                char name[256];
                snprintf(name, sizeof name, "./wf/q-%d-single.bin", done - 1);
                CHECK(ose_get_wavefield(h, OSE_FIELD_Q, field.data(), OSE_LAYOUT_YXZ));
                write_floats(name, field.data(), ncell);
                snprintf(name, sizeof name, "./wf/p-%d-single.bin", done - 1);
                CHECK(ose_get_wavefield(h, OSE_FIELD_P, field.data(), OSE_LAYOUT_YXZ));
                write_floats(name, field.data(), ncell);
            }
            printf("is=%d\tit=%d/%d\ttime=%f(s)/%f(s)\n", is, done, p.nt, p.dt * done, p.dt * p.nt);
        }
        CHECK(ose_write_outputs(h, "./output/qshot2.bin", nullptr));
    }
    CHECK(ose_write_outputs(h, nullptr, "./output/partest.txt"));
    ose_destroy(h);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    printf("finished: %f (s)\n", (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
    return 0;
}
