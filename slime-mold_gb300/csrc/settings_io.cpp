// settings_io.cpp - Settings (src/settings.rs:30-47) as text and files.
//
// The reference keeps its parameters only in memory (Settings::default()
// and the preset table); a settings file appears only as
// `simulation_settings.toml` in its .gitignore.  This file gives runs a
// reproducible parameter file in the TOML subset that the Settings struct
// maps onto field for field:
//
//   agent_count = 10000000
//   agent_possible_starting_headings = { start = 0.0, end = 360.0 }
//   window_fullscreen = false
//   pheromone_decay_factor = 10.0
//   ...
//
// Floats are written with 9 significant digits, which round-trips every
// binary32 value exactly, and always with a decimal point or an exponent
// (TOML's float syntax); inf and nan are written as TOML's `inf` / `nan`.
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "../../include/slime.h"

namespace {

enum Kind { kU64, kF32, kU32, kBool };

struct Field {
    const char* key;
    Kind kind;
    size_t offset;
};

// Settings' fields in the order of src/settings.rs:30-47; the heading range
// is written as one inline table and read through its two halves.
const Field kFields[] = {
    {"agent_count", kU64, offsetof(SlimeSettings, agent_count)},
    {"agent_jitter", kF32, offsetof(SlimeSettings, agent_jitter)},
    {"agent_speed_max", kF32, offsetof(SlimeSettings, agent_speed_max)},
    {"agent_speed_min", kF32, offsetof(SlimeSettings, agent_speed_min)},
    {"agent_turn_speed", kF32, offsetof(SlimeSettings, agent_turn_speed)},
    {"pheromone_decay_factor", kF32, offsetof(SlimeSettings, pheromone_decay_factor)},
    {"pheromone_diffusion_rate", kF32, offsetof(SlimeSettings, pheromone_diffusion_rate)},
    {"pheromone_deposition_amount", kF32, offsetof(SlimeSettings, pheromone_deposition_amount)},
    {"window_fullscreen", kBool, offsetof(SlimeSettings, window_fullscreen)},
    {"window_height", kU32, offsetof(SlimeSettings, window_height)},
    {"window_width", kU32, offsetof(SlimeSettings, window_width)},
    {"agent_sensor_angle", kF32, offsetof(SlimeSettings, agent_sensor_angle)},
    {"agent_sensor_distance", kF32, offsetof(SlimeSettings, agent_sensor_distance)},
    {"blur_radius", kF32, offsetof(SlimeSettings, blur_radius)},
    {"blur_sigma", kF32, offsetof(SlimeSettings, blur_sigma)},
};
constexpr const char* kHeadings = "agent_possible_starting_headings";

std::string float_text(float v) {
    if (isnan(v)) return "nan";
    if (isinf(v)) return v > 0 ? "inf" : "-inf";
    char b[64];
    snprintf(b, sizeof b, "%.9g", (double)v);
    std::string s = b;
    if (s.find_first_of(".en") == std::string::npos) s += ".0";
    return s;
}

std::string settings_text(const SlimeSettings& s) {
    std::string out = "# slime-mold settings (Settings, src/settings.rs:30-47)\n";
    const char* base = reinterpret_cast<const char*>(&s);
    for (const Field& f : kFields) {
        char b[96];
        const char* p = base + f.offset;
        switch (f.kind) {
        case kU64: {
            uint64_t v;
            memcpy(&v, p, 8);
            snprintf(b, sizeof b, "%llu", (unsigned long long)v);
            out += std::string(f.key) + " = " + b + "\n";
            break;
        }
        case kU32: {
            uint32_t v;
            memcpy(&v, p, 4);
            snprintf(b, sizeof b, "%u", v);
            out += std::string(f.key) + " = " + b + "\n";
            break;
        }
        case kBool: {
            uint32_t v;
            memcpy(&v, p, 4);
            out += std::string(f.key) + " = " + (v ? "true" : "false") + "\n";
            break;
        }
        case kF32: {
            float v;
            memcpy(&v, p, 4);
            out += std::string(f.key) + " = " + float_text(v) + "\n";
            break;
        }
        }
        if (strcmp(f.key, "agent_jitter") == 0)
            out += std::string(kHeadings) + " = { start = " + float_text(s.agent_possible_starting_headings_start) +
                   ", end = " + float_text(s.agent_possible_starting_headings_end) + " }\n";
    }
    return out;
}

std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r");
    return s.substr(a, b - a + 1);
}

// A TOML float (or integer, which a float field accepts): the whole token.
bool parse_f32(const std::string& t, float* out) {
    if (t == "nan" || t == "+nan" || t == "-nan") {
        *out = NAN;
        return true;
    }
    if (t == "inf" || t == "+inf") {
        *out = INFINITY;
        return true;
    }
    if (t == "-inf") {
        *out = -INFINITY;
        return true;
    }
    if (t.empty() || t.find_first_not_of("0123456789+-.eE_") != std::string::npos) return false;
    std::string u;
    for (char c : t)
        if (c != '_') u += c;
    errno = 0;
    char* end = nullptr;
    float v = strtof(u.c_str(), &end);
    if (end != u.c_str() + u.size() || errno == ERANGE) return false;
    *out = v;
    return true;
}

bool parse_uint(const std::string& t, uint64_t max, uint64_t* out) {
    if (t.empty() || t.find_first_not_of("0123456789_") != std::string::npos || t[0] == '_') return false;
    uint64_t v = 0;
    for (char c : t) {
        if (c == '_') continue;
        uint64_t d = (uint64_t)(c - '0');
        if (v > (max - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = v;
    return true;
}

// `{ start = a, end = b }`
bool parse_range(const std::string& t, float* start, float* end) {
    if (t.size() < 2 || t.front() != '{' || t.back() != '}') return false;
    std::string body = t.substr(1, t.size() - 2);
    bool have_s = false, have_e = false;
    size_t pos = 0;
    while (pos <= body.size()) {
        size_t comma = body.find(',', pos);
        std::string item = trim(body.substr(pos, comma == std::string::npos ? std::string::npos : comma - pos));
        size_t eq = item.find('=');
        if (eq == std::string::npos) return false;
        std::string k = trim(item.substr(0, eq)), v = trim(item.substr(eq + 1));
        if (k == "start" && !have_s) {
            if (!parse_f32(v, start)) return false;
            have_s = true;
        } else if (k == "end" && !have_e) {
            if (!parse_f32(v, end)) return false;
            have_e = true;
        } else {
            return false;
        }
        if (comma == std::string::npos) break;
        pos = comma + 1;
    }
    return have_s && have_e;
}

// Strip a trailing comment that is not inside the value's braces.
std::string strip_comment(const std::string& line) {
    size_t h = line.find('#');
    return h == std::string::npos ? line : line.substr(0, h);
}

int parse_settings(const char* text, SlimeSettings* out, int* error_line) {
    SlimeSettings s;
    slime_settings_default(&s);
    char* base = reinterpret_cast<char*>(&s);
    bool seen[sizeof(kFields) / sizeof(kFields[0]) + 1] = {};
    int lineno = 0;
    const char* p = text;
    while (*p) {
        const char* nl = strchr(p, '\n');
        std::string line = nl ? std::string(p, nl - p) : std::string(p);
        p = nl ? nl + 1 : p + strlen(p);
        lineno++;
        line = trim(strip_comment(line));
        if (line.empty()) continue;
        size_t eq = line.find('=');
        if (eq == std::string::npos) goto bad;
        {
            std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
            if (key == kHeadings) {
                const size_t idx = sizeof(kFields) / sizeof(kFields[0]);
                if (seen[idx] || !parse_range(val, &s.agent_possible_starting_headings_start,
                                              &s.agent_possible_starting_headings_end))
                    goto bad;
                seen[idx] = true;
                continue;
            }
            size_t i = 0;
            for (; i < sizeof(kFields) / sizeof(kFields[0]); i++)
                if (key == kFields[i].key) break;
            if (i == sizeof(kFields) / sizeof(kFields[0]) || seen[i]) goto bad;
            seen[i] = true;
            char* dst = base + kFields[i].offset;
            switch (kFields[i].kind) {
            case kU64: {
                uint64_t v;
                if (!parse_uint(val, UINT64_MAX, &v)) goto bad;
                memcpy(dst, &v, 8);
                break;
            }
            case kU32: {
                uint64_t v;
                if (!parse_uint(val, UINT32_MAX, &v)) goto bad;
                uint32_t w = (uint32_t)v;
                memcpy(dst, &w, 4);
                break;
            }
            case kBool: {
                uint32_t w;
                if (val == "true") w = 1;
                else if (val == "false") w = 0;
                else goto bad;
                memcpy(dst, &w, 4);
                break;
            }
            case kF32: {
                float v;
                if (!parse_f32(val, &v)) goto bad;
                memcpy(dst, &v, 4);
                break;
            }
            }
            continue;
        }
    bad:
        if (error_line) *error_line = lineno;
        return SLIME_ERR_INVALID_ARGUMENT;
    }
    if (error_line) *error_line = 0;
    *out = s;
    return SLIME_OK;
}

} // namespace

extern "C" {

int slime_settings_to_text(const SlimeSettings* s, char* buf, size_t cap, size_t* len) {
    if (!s || (!buf && cap)) return SLIME_ERR_INVALID_ARGUMENT;
    const std::string t = settings_text(*s);
    if (len) *len = t.size();
    if (cap < t.size() + 1) return SLIME_ERR_INVALID_ARGUMENT;
    memcpy(buf, t.c_str(), t.size() + 1);
    return SLIME_OK;
}

int slime_settings_from_text(const char* text, SlimeSettings* out, int* error_line) {
    if (error_line) *error_line = 0;
    if (!text || !out) return SLIME_ERR_INVALID_ARGUMENT;
    return parse_settings(text, out, error_line);
}

int slime_settings_save(const SlimeSettings* s, const char* path) {
    if (!s || !path) return SLIME_ERR_INVALID_ARGUMENT;
    const std::string t = settings_text(*s);
    FILE* f = fopen(path, "wb");
    if (!f) return SLIME_ERR_INVALID_ARGUMENT;
    const bool ok = fwrite(t.data(), 1, t.size(), f) == t.size();
    return (fclose(f) == 0 && ok) ? SLIME_OK : SLIME_ERR_INVALID_ARGUMENT;
}

int slime_settings_load(const char* path, SlimeSettings* out, int* error_line) {
    if (error_line) *error_line = 0;
    if (!path || !out) return SLIME_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "rb");
    if (!f) return SLIME_ERR_INVALID_ARGUMENT;
    std::string t;
    char b[4096];
    size_t k;
    while ((k = fread(b, 1, sizeof b, f)) > 0) t.append(b, k);
    const bool err = ferror(f) != 0;
    fclose(f);
    if (err || t.find('\0') != std::string::npos) return SLIME_ERR_INVALID_ARGUMENT;
    return parse_settings(t.c_str(), out, error_line);
}

} // extern "C"
