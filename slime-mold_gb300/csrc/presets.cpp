// presets.cpp - the reference's parameter surface: Settings::default()
// (src/settings.rs:49-70), the preset table of init_preset_manager()
// (src/presets.rs:45-155) and SimSizeUniform::new (src/main.rs:48-66).
#include <string.h>

#include "../../include/slime.h"

namespace {

// Constants of src/settings.rs:4-27.
constexpr uint32_t kDefaultWidth = 1600;
constexpr uint32_t kDefaultHeight = 900;
constexpr uint64_t kAgentCount = 10000000;
constexpr float kAgentSpeedMin = 30.0f;
constexpr float kAgentSpeedMax = 50.0f;
constexpr float kAgentTurnSpeed = 0.43f;
constexpr float kDepositionAmount = 1.0f;
constexpr float kAgentJitter = 0.0f;
constexpr float kAgentSensorAngle = 0.3f;
constexpr float kAgentSensorDistance = 20.0f;
constexpr float kDecayFactor = 10.0f;
constexpr float kDiffusionRate = 1.0f;
constexpr float kBlurRadius = 2.0f;
constexpr float kBlurSigma = 1.0f;

SlimeSettings defaults() {
    SlimeSettings s;
    memset(&s, 0, sizeof(s));
    s.agent_count = kAgentCount;
    s.agent_jitter = kAgentJitter;
    s.agent_possible_starting_headings_start = 0.0f; // AGENT_POSSIBLE_STARTING_HEADINGS = 0.0..360.0
    s.agent_possible_starting_headings_end = 360.0f;
    s.agent_speed_max = kAgentSpeedMax;
    s.agent_speed_min = kAgentSpeedMin;
    s.agent_turn_speed = kAgentTurnSpeed;
    s.pheromone_decay_factor = kDecayFactor;
    s.pheromone_diffusion_rate = kDiffusionRate;
    s.pheromone_deposition_amount = kDepositionAmount;
    s.window_fullscreen = 0;
    s.window_height = kDefaultHeight;
    s.window_width = kDefaultWidth;
    s.agent_sensor_angle = kAgentSensorAngle;
    s.agent_sensor_distance = kAgentSensorDistance;
    s.blur_radius = kBlurRadius;
    s.blur_sigma = kBlurSigma;
    return s;
}

struct PresetRow {
    const char* name;
    bool is_default;
    uint64_t agent_count; // 0 = keep the default
    float jitter, speed_min, speed_max, turn, sensor_angle, sensor_distance, deposition, decay, diffusion;
};

// src/presets.rs:47-153, in insertion order.
const PresetRow kPresets[] = {
    {"Default", true, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {"Sponge", false, 0, 0.0f, 20.0f, 30.0f, 0.43f, 0.3f, 20.0f, 1.0f, 1.0f, 1.0f},
    {"Firecracker Trees", false, 0, 0.1f, 60.0f, 60.0f, 1.47f, 0.3f, 20.0f, 1.0f, 10.0f, 1.0f},
    {"Threads", false, 0, 0.0f, 70.0f, 80.0f, 0.02f, 0.3f, 20.0f, 1.0f, 10.0f, 0.1f},
    {"Curls", false, 3000000, 5.0f, 70.0f, 80.0f, 0.05f, 0.3f, 20.0f, 1.0f, 75.0f, 0.1f},
    {"Waves", false, 0, 1.0f, 30.0f, 50.0f, 6.0f, 0.3f, 20.0f, 1.0f, 10.0f, 0.1f},
    {"Snake", false, 0, 3.0f, 100.0f, 120.0f, 0.37f, 1.34f, 225.0f, 1.0f, 10.0f, 1.0f},
    {"Mesh", false, 0, 3.0f, 100.0f, 120.0f, 6.0f, 1.57f, 225.0f, 1.0f, 10.0f, 1.0f},
};
constexpr int kNumPresets = (int)(sizeof(kPresets) / sizeof(kPresets[0]));

SlimeSettings from_row(const PresetRow& r) {
    SlimeSettings s = defaults();
    if (r.is_default) return s;
    if (r.agent_count) s.agent_count = r.agent_count;
    s.agent_jitter = r.jitter;
    s.agent_speed_min = r.speed_min;
    s.agent_speed_max = r.speed_max;
    s.agent_turn_speed = r.turn;
    s.agent_sensor_angle = r.sensor_angle;
    s.agent_sensor_distance = r.sensor_distance;
    s.pheromone_deposition_amount = r.deposition;
    s.pheromone_decay_factor = r.decay;
    s.pheromone_diffusion_rate = r.diffusion;
    return s;
}

} // namespace

extern "C" {

void slime_settings_default(SlimeSettings* out) {
    if (out) *out = defaults();
}

int slime_preset_count(void) { return kNumPresets; }

int slime_preset_get(int index, const char** name, SlimeSettings* out) {
    if (index < 0 || index >= kNumPresets) return SLIME_ERR_INVALID_ARGUMENT;
    if (name) *name = kPresets[index].name;
    if (out) *out = from_row(kPresets[index]);
    return SLIME_OK;
}

int slime_preset_find(const char* name, SlimeSettings* out) {
    if (!name) return SLIME_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < kNumPresets; i++)
        if (strcmp(kPresets[i].name, name) == 0) {
            if (out) *out = from_row(kPresets[i]);
            return SLIME_OK;
        }
    return SLIME_ERR_INVALID_ARGUMENT;
}

void slime_params_from_settings(const SlimeSettings* s, uint32_t width, uint32_t height, SlimeParams* out) {
    if (!s || !out) return;
    memset(out, 0, sizeof(*out));
    out->width = width;
    out->height = height;
    out->decay_factor = s->pheromone_decay_factor;
    out->agent_jitter = s->agent_jitter;
    out->agent_speed_min = s->agent_speed_min;
    out->agent_speed_max = s->agent_speed_max;
    out->agent_turn_speed = s->agent_turn_speed;
    out->agent_sensor_angle = s->agent_sensor_angle;
    out->agent_sensor_distance = s->agent_sensor_distance;
    out->diffusion_rate = s->pheromone_diffusion_rate;
    out->pheromone_deposition_amount = s->pheromone_deposition_amount;
    out->blur_radius = s->blur_radius;
    out->blur_sigma = s->blur_sigma;
    out->_pad = 0;
    out->time_step = 0.016f; // TIME_STEP, compute.wgsl:55
    out->decay_mode = SLIME_DECAY_REF_SUBTRACT;
    out->blur_mode = SLIME_BLUR_REF_BOX3;
    out->dispatch_mode = SLIME_DISPATCH_EACH_AGENT;
    out->sensor_mode = SLIME_SENSOR_SHADER; // cos/sin(angle -/+ a), compute.wgsl:75-86
}

} // extern "C"
