// sc_run -- a spatial_cell_sim-style driver of libspatialcell (C++ on the C ABI).
//
// The reference's executable is main() in spatial_cell_sim/src/main.cu:142-721:
// it reads ./config.json and the tables in ../universe-config/gen, sets up a
// scene on the host, steps `steps` times and appends every
// persistEveryNthFrame-th reduced frame to ./results/frames.dat.  This driver
// does the same through the library: config.json (sc_config_load_json, with
// the extension keys), the type and rule tables (sc_types_load_json /
// sc_rules_load_json), a scene generated on the device (sc_generate_uniform:
// particles of the given type mix uniform in the box; the reference's
// hand-built demo scene of setup/setup.cuh is not part of the step), then
// sc_prepare, sc_step and the frames streamed to frames.dat while the next
// steps run (sc_reduce_frame_async into two pinned slots).
//
//   sc_run [--config config.json] [--types large-molecules.json]
//          [--rules complexification.json] [--frames results/frames.dat]
//          [--steps N] [--particles N] [--metabolic N]
//          [--mix type:fraction,...] [--seed S]
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "spatialcell.h"

namespace {

void usage() {
    fprintf(stderr,
            "usage: sc_run [--config config.json] [--types large-molecules.json] [--rules complexification.json]\n"
            "              [--frames results/frames.dat] [--steps N] [--particles N] [--metabolic N]\n"
            "              [--mix type:fraction,...] [--seed S]\n");
}

int fail(const char *what, const sc_sim *sim) {
    fprintf(stderr, "sc_run: %s: %s\n", what, sc_last_error(sim));
    return 1;
}

}  // namespace

int main(int argc, char **argv) {
    std::string configPath = "./config.json", typesPath = "../universe-config/gen/large-molecules.json",
                rulesPath = "../universe-config/gen/complexification.json", framesPath = "./results/frames.dat";
    long steps = -1, particles = -1, metabolic = -1;
    unsigned long long seed = 42;
    std::vector<int32_t> kinds;
    std::vector<float> fractions;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--help" || a == "-h") { usage(); return 0; }
        if (i + 1 >= argc) { usage(); return 2; }
        const char *v = argv[++i];
        if (a == "--config") configPath = v;
        else if (a == "--types") typesPath = v;
        else if (a == "--rules") rulesPath = v;
        else if (a == "--frames") framesPath = v;
        else if (a == "--steps") steps = atol(v);
        else if (a == "--particles") particles = atol(v);
        else if (a == "--metabolic") metabolic = atol(v);
        else if (a == "--seed") seed = strtoull(v, nullptr, 10);
        else if (a == "--mix") {
            std::string s = v;
            size_t p = 0;
            while (p < s.size()) {
                size_t e = s.find(',', p);
                std::string item = s.substr(p, e == std::string::npos ? std::string::npos : e - p);
                size_t c = item.find(':');
                if (c == std::string::npos) { usage(); return 2; }
                kinds.push_back(atoi(item.substr(0, c).c_str()));
                fractions.push_back((float)atof(item.substr(c + 1).c_str()));
                p = e == std::string::npos ? s.size() : e + 1;
            }
        } else { usage(); return 2; }
    }

    sc_config cfg;
    sc_config_defaults(&cfg);
    if (sc_config_load_json(configPath.c_str(), &cfg)) return fail("config", nullptr);  // Config(Json::Value)
    if (steps >= 0) cfg.steps = (int32_t)steps;
    int32_t nt = 0, nr = 0;
    if (sc_types_load_json(typesPath.c_str(), nullptr, 0, &nt)) return fail("type table", nullptr);
    std::vector<sc_type_info> types((size_t)nt);
    if (sc_types_load_json(typesPath.c_str(), types.data(), nt, &nt)) return fail("type table", nullptr);
    if (sc_rules_load_json(rulesPath.c_str(), nullptr, 0, &nr)) return fail("rule table", nullptr);
    std::vector<sc_rule> rules((size_t)nr);
    if (sc_rules_load_json(rulesPath.c_str(), rules.data(), nr, &nr)) return fail("rule table", nullptr);
    if (kinds.empty()) { kinds = {0}; fractions = {1.0f}; }

    sc_sim *sim = nullptr;
    if (sc_create(&cfg, types.data(), nt, rules.data(), nr, &sim)) return fail("create", nullptr);
    const int32_t n = particles >= 0 ? (int32_t)particles : cfg.num_particles;
    const int32_t nm = metabolic >= 0 ? (int32_t)metabolic : cfg.num_metabolic_particles;
    if (sc_generate_uniform(sim, n, nm, kinds.data(), fractions.data(), (int32_t)kinds.size(), seed))
        return fail("scene", sim);
    if (sc_prepare(sim)) return fail("prepare", sim);  // main.cu:284-338

    FILE *frames = fopen(framesPath.c_str(), "wb");
    if (!frames) { fprintf(stderr, "sc_run: cannot open %s\n", framesPath.c_str()); return 1; }
    if (sc_frames_write_header(frames, &cfg)) return fail("frames.dat header", nullptr);
    // two pinned frame slots: frame k lands in slot k % 2 while the next steps run
    const size_t rpBytes = (size_t)cfg.num_particles * sizeof(sc_reduced_particle);
    const size_t rmBytes = (size_t)cfg.num_metabolic_particles * sizeof(sc_reduced_metabolic_particle);
    sc_reduced_particle *rp[2];
    sc_reduced_metabolic_particle *rm[2];
    for (int k = 0; k < 2; k++) {
        if (cudaHostAlloc((void **)&rp[k], rpBytes ? rpBytes : 1, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void **)&rm[k], rmBytes ? rmBytes : 1, cudaHostAllocDefault) != cudaSuccess) {
            fprintf(stderr, "sc_run: pinned host memory\n");
            return 1;
        }
    }
    int64_t ticket[2] = {-1, -1};
    int slot = 0;
    auto write_slot = [&](int k) -> int {  // writes the frame of slot k once it has landed
        if (ticket[k] < 0) return 0;
        if (sc_frame_wait(sim, ticket[k])) return fail("frame", sim);
        if (sc_frames_write_frame(frames, &cfg, rp[k], rm[k])) return fail("frames.dat", nullptr);
        ticket[k] = -1;
        return 0;
    };
    auto persist = [&]() -> int {  // persistFrame, main.cu:95-126
        if (write_slot(slot)) return 1;
        ticket[slot] = sc_reduce_frame_async(sim, rp[slot], rm[slot]);
        if (ticket[slot] < 0) return fail("frame", sim);
        slot ^= 1;
        return 0;
    };
    if (persist()) return 1;  // frame 0, main.cu:314-322
    const int every = cfg.persist_every_nth_frame > 0 ? cfg.persist_every_nth_frame : 1;
    auto t0 = std::chrono::steady_clock::now();
    for (int step = 0; step < cfg.steps; step++) {
        if (sc_step(sim, 1)) return fail("step", sim);  // main.cu:347-661
        if (step % every == 0 && persist()) return 1;
        if (cfg.report_every_nth_frame > 0 && step % cfg.report_every_nth_frame == 0) {
            sc_counters c;
            if (sc_get_counters(sim, &c)) return fail("counters", sim);
            printf("step %d, nActiveParticles %d\n", step, c.n_active_particles);
        }
    }
    if (write_slot(slot) || write_slot(slot ^ 1)) return 1;
    if (sc_sync(sim)) return fail("sync", sim);
    double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("time %f\n", s);
    fclose(frames);
    for (int k = 0; k < 2; k++) {
        cudaFreeHost(rp[k]);
        cudaFreeHost(rm[k]);
    }
    sc_destroy(sim);
    printf("Done\n");
    return 0;
}
