// sc_host.cpp -- host side of the setup surface: config.json, the type and
// rule tables, and the frames.dat writer.
//
// config.json keys and the grid derivation follow config.cuh:15-75;
// large-molecules.json follows loadParticleTypeInfo / flattenParticleTypeInfo
// (chemistry.cuh:10-51); complexification.json follows
// loadComplexificationInfo (interactions.cuh:17-54), whose jsoncpp calls give
// these rules: a missing key takes the default of interactions.cuh:33-49, an
// explicit null reads as 0 / false (jsoncpp's asInt() / asBool() of null), a
// real literal read as int is truncated, and float fields are the double
// value rounded to float.  frames.dat follows FileStorage (storage.cuh:22-39).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "sc_json.hpp"
#include "spatialcell.h"

namespace {

thread_local std::string g_host_error;

int fail(int code, const std::string &msg) {
    g_host_error = msg;
    return code;
}

bool read_json(const char *path, scjson::Value &v, int *rc) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { *rc = fail(SC_E_IO, std::string("cannot open ") + path); return false; }
    std::stringstream ss;
    ss << f.rdbuf();
    std::string err;
    if (!scjson::parse(ss.str(), v, err)) { *rc = fail(SC_E_PARSE, std::string(path) + ": " + err); return false; }
    return true;
}

// jsoncpp conversions (Value::asInt / asFloat / asBool)
int as_int(const scjson::Value *v) {
    if (!v) return 0;
    switch (v->type) {
        case scjson::Value::Bool: return v->b ? 1 : 0;
        case scjson::Value::Int: return (int)v->i;
        case scjson::Value::Real: return (int)v->d;
        default: return 0;
    }
}
float as_float(const scjson::Value *v) { return v ? (float)v->as_double() : 0.0f; }
bool as_bool(const scjson::Value *v) {
    if (!v) return false;
    switch (v->type) {
        case scjson::Value::Bool: return v->b;
        case scjson::Value::Int: return v->i != 0;
        case scjson::Value::Real: return v->d != 0.0;
        default: return false;
    }
}
// c.get(key, default): the member if present (even an explicit null), else the default
int get_int(const scjson::Value &o, const char *k, int def) {
    const scjson::Value *m = o.find(k);
    return m ? as_int(m) : def;
}
bool get_bool(const scjson::Value &o, const char *k, bool def) {
    const scjson::Value *m = o.find(k);
    return m ? as_bool(m) : def;
}
float get_float(const scjson::Value &o, const char *k, double def) {
    const scjson::Value *m = o.find(k);
    return m ? as_float(m) : (float)def;
}
const scjson::Value *elem(const scjson::Value *a, size_t i) {
    return (a && a->type == scjson::Value::Array && i < a->arr.size()) ? &a->arr[i] : nullptr;
}

}  // namespace

extern "C" const char *sc_host_last_error(void) { return g_host_error.c_str(); }

extern "C" void sc_config_defaults(sc_config *c) {
    memset(c, 0, sizeof *c);
    c->num_particles = 65536;
    c->num_metabolic_particles = 65536;
    c->steps = 401;
    c->sim_size = 400.0f;
    c->max_interaction_distance = 8.0f;
    c->max_diffusion_distance = 10.0f;
    c->grid_cell_size = 10.0f;
    c->movement_noise_scale = 0.7f;
    c->rotation_noise_scale = 0.05f;
    c->metabolite_movement_noise_scale = 1.5f;
    c->velocity_decay = 0.7f;
    c->angular_velocity_decay = 0.7f;
    c->noise_coordination_steps = 16;
    c->relaxation_steps = 32;
    c->metabolite_diffusion_steps = 8;
    c->persist_every_nth_frame = 1;
    c->report_every_nth_frame = 10;
    c->num_metabolites = SC_AOS_NUM_METABOLITES;
    c->seed = 42;
    c->graphs = 1;
    c->class_streams = 0;
    c->tiles = 0;
    c->pair_list_limit = -1;
    c->pool_per_item = -1;
    c->pair_claim = 0;
    c->rule_probabilities = 0;
    c->metabolic_pairs = 1;
    c->propagate_state = 0;
}

extern "C" int sc_config_load_json(const char *path, sc_config *c) {
    if (!path || !c) return fail(SC_E_INVALID, "null argument");
    scjson::Value v;
    int rc = SC_OK;
    if (!read_json(path, v, &rc)) return rc;
    if (v.type != scjson::Value::Object) return fail(SC_E_PARSE, "config.json is not an object");
    auto I = [&](const char *k, int32_t *dst) { if (const scjson::Value *m = v.find(k)) *dst = as_int(m); };
    auto F = [&](const char *k, float *dst) { if (const scjson::Value *m = v.find(k)) *dst = as_float(m); };
    I("numParticles", &c->num_particles);
    I("numMetabolicParticles", &c->num_metabolic_particles);
    I("steps", &c->steps);
    F("simSize", &c->sim_size);
    F("maxInteractionDistance", &c->max_interaction_distance);
    F("maxDiffusionDistance", &c->max_diffusion_distance);
    F("gridCellSize", &c->grid_cell_size);
    F("movementNoiseScale", &c->movement_noise_scale);
    F("rotationNoiseScale", &c->rotation_noise_scale);
    F("metaboliteMovementNoiseScale", &c->metabolite_movement_noise_scale);
    F("velocityDecay", &c->velocity_decay);
    F("angularVelocityDecay", &c->angular_velocity_decay);
    I("noiseCoordinationSteps", &c->noise_coordination_steps);
    I("relaxationSteps", &c->relaxation_steps);
    I("metaboliteDiffusionSteps", &c->metabolite_diffusion_steps);
    I("persistEveryNthFrame", &c->persist_every_nth_frame);
    I("reportEveryNthFrame", &c->report_every_nth_frame);
    I("numMetabolites", &c->num_metabolites);
    I("periodic", &c->periodic);
    I("walls", &c->walls);
    I("pairClaim", &c->pair_claim);
    I("ruleProbabilities", &c->rule_probabilities);
    I("propagateState", &c->propagate_state);
    if (const scjson::Value *m = v.find("seed")) c->seed = (uint64_t)(m->type == scjson::Value::Int ? m->i : (long long)m->as_double());
    return SC_OK;
}

extern "C" int sc_config_grid(const sc_config *c, int32_t *n_grid_cells, int32_t *n_grid_bits) {
    if (!c || !(c->grid_cell_size > 0.0f) || !(c->sim_size > 0.0f)) return fail(SC_E_INVALID, "bad grid configuration");
    float q = ceilf(c->sim_size / c->grid_cell_size);
    if (!(q < 1024.0f)) return fail(SC_E_INVALID, "more than 1024 grid cells per axis");
    int n = (int)q, bits = 1, p2 = 2;
    while (p2 < n) { p2 *= 2; bits++; }
    if (n_grid_cells) *n_grid_cells = p2;
    if (n_grid_bits) *n_grid_bits = bits;
    return SC_OK;
}

extern "C" int sc_types_load_json(const char *path, sc_type_info *out, int32_t capacity, int32_t *n_types) {
    scjson::Value v;
    int rc = SC_OK;
    if (!read_json(path, v, &rc)) return rc;
    if (v.type != scjson::Value::Array) return fail(SC_E_PARSE, "type table is not an array");
    int maxType = 0;
    for (const auto &m : v.arr) maxType = std::max(maxType, as_int(m.find("type")));
    if (n_types) *n_types = maxType + 1;
    if (!out) return SC_OK;
    if (capacity < maxType + 1) return fail(SC_E_INVALID, "type table capacity too small");
    memset(out, 0, sizeof(sc_type_info) * (size_t)(maxType + 1));
    // std::unordered_map::insert keeps the first entry of a repeated type
    std::vector<char> seen((size_t)maxType + 1, 0);
    for (const auto &m : v.arr) {
        int t = as_int(m.find("type"));
        if (t < 0 || seen[(size_t)t]) continue;
        seen[(size_t)t] = 1;
        out[t].radius = as_float(m.find("radius"));
        out[t].hydrophobic = (int8_t)get_int(m, "hydrophobic", 0);
    }
    return SC_OK;
}

extern "C" int sc_rules_load_json(const char *path, sc_rule *out, int32_t capacity, int32_t *n_rules) {
    scjson::Value v;
    int rc = SC_OK;
    if (!read_json(path, v, &rc)) return rc;
    if (v.type != scjson::Value::Array) return fail(SC_E_PARSE, "rule table is not an array");
    if (n_rules) *n_rules = (int32_t)v.arr.size();
    if (!out) return SC_OK;
    if ((size_t)capacity < v.arr.size()) return fail(SC_E_INVALID, "rule table capacity too small");
    for (size_t i = 0; i < v.arr.size(); i++) {
        const scjson::Value &c = v.arr[i];
        sc_rule &r = out[i];
        memset(&r, 0, sizeof r);
        r.id = as_int(c.find("id"));
        r.group = get_int(c, "group", -1);
        r.first_partner_type = as_int(c.find("firstPartnerType"));
        r.first_partner_state = (int8_t)get_int(c, "firstPartnerState", -1);
        r.second_partner_type = as_int(c.find("secondPartnerType"));
        r.second_partner_state = (int8_t)get_int(c, "secondPartnerState", -1);
        r.propagate_state = get_bool(c, "propagateState", false);
        r.set_state = get_bool(c, "setState", true);
        r.wait_for_state = get_bool(c, "waitForState", true);
        r.wait_for_alignment = get_bool(c, "waitForAlignment", true);
        r.only_via_transition = get_bool(c, "onlyViaTransition", false);
        r.transition_to = get_int(c, "transitionTo", -1);
        r.polymerize = get_int(c, "polymerize", -1);
        r.break_after_transition = get_bool(c, "breakAfterTransition", false);
        const scjson::Value *ro = c.find("relativeOrientation"), *rp = c.find("relativePosition");
        for (int k = 0; k < 4; k++) r.relative_orientation[k] = as_float(elem(ro, (size_t)k));
        r.orientation_alignment_threshold = get_float(c, "orientationAlignmentThreshold", 0.8);
        for (int k = 0; k < 3; k++) r.relative_position[k] = as_float(elem(rp, (size_t)k));
        r.position_alignment_threshold = get_float(c, "positionAlignmentThreshold", 0.8);
        // extension key (not read by the reference): a per-step binding probability
        if (const scjson::Value *pr = c.find("probability")) {
            r.use_probability = 1;
            r.probability = as_float(pr);
        }
    }
    return SC_OK;
}

// storage.cuh:22-27: f32 simSize, u32 numParticles, u32 numMetabolicParticles
extern "C" int sc_frames_write_header(void *file, const sc_config *c) {
    FILE *f = (FILE *)file;
    if (!f || !c) return fail(SC_E_INVALID, "null argument");
    uint32_t n = (uint32_t)c->num_particles, nm = (uint32_t)c->num_metabolic_particles;
    if (fwrite(&c->sim_size, 4, 1, f) != 1 || fwrite(&n, 4, 1, f) != 1 || fwrite(&nm, 4, 1, f) != 1)
        return fail(SC_E_IO, "frames.dat header write failed");
    return SC_OK;
}

// storage.cuh:29-39: u32 count, records (capacity-sized), for both sets
extern "C" int sc_frames_write_frame(void *file, const sc_config *c, const sc_reduced_particle *p,
                                     const sc_reduced_metabolic_particle *m) {
    FILE *f = (FILE *)file;
    if (!f || !c || !p || !m) return fail(SC_E_INVALID, "null argument");
    uint32_t n = (uint32_t)c->num_particles, nm = (uint32_t)c->num_metabolic_particles;
    if (fwrite(&n, 4, 1, f) != 1 || fwrite(p, sizeof *p, n, f) != n || fwrite(&nm, 4, 1, f) != 1 ||
        fwrite(m, sizeof *m, nm, f) != nm)
        return fail(SC_E_IO, "frames.dat frame write failed");
    return SC_OK;
}
