/*
 * slime_oracle.cpp - CPU oracle for the Physarum step.  TEST INFRASTRUCTURE:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, always as the checker or as the timed CPU baseline, never as
 * part of the product path.
 *
 * PINNED AGAINST THE REFERENCE'S OWN SHADER.  The reference (Velfi/slime-mold)
 * has no tests, golden vectors or fixtures, and its Rust/wgpu program cannot
 * run here.  This file is a line-by-line binary32 restatement of
 * src/compute.wgsl; oracle/wgsl/ translates that shader mechanically to C++
 * and runs it invocation by invocation, and tests/test_reference_pin.py and
 * the frames in tests/golden/wgsl/ show this restatement equal to it bit for
 * bit (sampler, decay, diffuse, agent update at any sensor angle, whole
 * frames where the shader does not race).  The opt-in SLIME_SENSOR_ROTATED
 * mode is the one deliberate difference: its side sensors' directions are
 * rotations of the centre direction, a few ulp from the shader's cos/sin of
 * the shifted angle.  Also checked against hand-derived known answers and an
 * independent pure-Python restatement (tests/golden).
 *
 * What it restates:
 *   sample_trail_map       compute.wgsl:7-29
 *   agent update "main"    compute.wgsl:57-145
 *   decay_trail            compute.wgsl:148-161
 *   diffuse_trail          compute.wgsl:164-195
 * with the WGSL builtins taken from include/slime_math.h, and with defined
 * semantics where the shader races (sensing reads the pre-step trail; the k
 * deposits into a cell are folded sequentially; decay+diffuse read one buffer
 * and write another; every agent is updated once per step).
 *
 * It also holds binary64 twins of the trail pass and of the frozen-trajectory
 * deposit -> decay -> diffuse chain with its hand-derived adjoint, used to
 * state the binary32 error and to check the GPU gradients.
 *
 * Build: oracle/build_oracle.py (g++ -O3 -ffp-contract=off -fopenmp).  The
 * -ffp-contract=off flag is required: the restatement must not fuse a*b+c.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../include/slime.h"
#include "../include/slime_math.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* sample_trail_map, compute.wgsl:7-29. */
inline float sample_trail_map(const float* trail, int32_t W, int32_t H, float px, float py) {
    int32_t x0 = slm_f2i(slm_floor(px));
    int32_t y0 = slm_f2i(slm_floor(py));
    /* x1 = x0 + 1 >= W is written as x0 >= W - 1 so that a saturated x0 cannot
     * wrap around (compute.wgsl:10-16). */
    if (x0 < 0 || x0 >= W - 1 || y0 < 0 || y0 >= H - 1) return 0.0f;
    int32_t x1 = x0 + 1;
    int32_t y1 = y0 + 1;
    float dx = slm_sub(px, slm_i2f(x0));
    float dy = slm_sub(py, slm_i2f(y0));
    float v00 = trail[y0 * W + x0];
    float v10 = trail[y0 * W + x1];
    float v01 = trail[y1 * W + x0];
    float v11 = trail[y1 * W + x1];
    float v0 = slm_mix(v00, v10, dx);
    float v1 = slm_mix(v01, v11, dx);
    return slm_mix(v0, v1, dy);
}

/* The three sensor samples of compute.wgsl:75-95 for an agent at (x, y)
 * heading `angle`: sensor angles angle - a, angle + a, angle (:75-77) and
 * their cos/sin (:79-90), each evaluated as written (slm_sensor_dirs_shader);
 * with SLIME_SENSOR_ROTATED the side directions are the centre direction's
 * rotations by -a and +a instead (slm_sensor_dirs). */
inline void sense(const SlimeParams* p, int32_t W, int32_t H, float x, float y, float angle, const float* trail,
                  float* left_value, float* right_value, float* center_value) {
    float dist = p->agent_sensor_distance;
    float sl, cl, sr, cr, sc, cc;
    if (p->sensor_mode == SLIME_SENSOR_ROTATED) {
        float sa, ca;
        slm_sincos(p->agent_sensor_angle, &sa, &ca);
        slm_sensor_dirs(angle, sa, ca, &cl, &sl, &cc, &sc, &cr, &sr);
    } else {
        slm_sensor_dirs_shader(angle, p->agent_sensor_angle, &cl, &sl, &cc, &sc, &cr, &sr);
    }
    float lpx = slm_add(x, slm_mul(dist, cl)); /* :79-82 */
    float lpy = slm_add(y, slm_mul(dist, sl));
    float rpx = slm_add(x, slm_mul(dist, cr)); /* :83-86 */
    float rpy = slm_add(y, slm_mul(dist, sr));
    float cpx = slm_add(x, slm_mul(dist, cc)); /* :87-90 */
    float cpy = slm_add(y, slm_mul(dist, sc));
    *left_value = sample_trail_map(trail, W, H, lpx, lpy);   /* :93 */
    *right_value = sample_trail_map(trail, W, H, rpx, rpy);  /* :94 */
    *center_value = sample_trail_map(trail, W, H, cpx, cpy); /* :95 */
}

/* The agent invocation "main", compute.wgsl:57-145, for agent `index`.
 * Returns the deposit cell or -1. */
inline int64_t agent_update(const SlimeParams* p, int32_t W, int32_t H, int32_t index, float* a,
                            const float* trail) {
    float x = a[0];
    float y = a[1];
    float angle = a[2];
    float speed = a[3];

    speed = slm_clamp(speed, p->agent_speed_min, p->agent_speed_max); /* :72 */

    float left_value, right_value, center_value;
    sense(p, W, H, x, y, angle, trail, &left_value, &right_value, &center_value);

    if (center_value > left_value && center_value > right_value) { /* :98 */
        /* continue straight */
    } else if (left_value > right_value) { /* :100-104 */
        float target_angle = slm_sub(angle, SLM_WGSL_TAU);
        float angle_diff = slm_sub(target_angle, angle);
        angle = slm_add(angle, slm_mul(slm_min(p->agent_turn_speed, slm_abs(angle_diff)), slm_sign(angle_diff)));
    } else if (right_value > left_value) { /* :105-109 */
        float target_angle = slm_add(angle, SLM_WGSL_TAU);
        float angle_diff = slm_sub(target_angle, angle);
        angle = slm_add(angle, slm_mul(slm_min(p->agent_turn_speed, slm_abs(angle_diff)), slm_sign(angle_diff)));
    }

    /* jitter, :115-118, from the pre-move x, y and the agent's index */
    float random_val = slm_jitter_hash(index, x, y);
    angle = slm_add(angle, slm_mul(slm_sub(slm_mul(random_val, 2.0f), 1.0f), p->agent_jitter));

    angle = slm_fmod(angle, SLM_WGSL_TWO_PI); /* :121-122 */
    if (angle < 0.0f) angle = slm_add(angle, SLM_WGSL_TWO_PI);

    float move_dist = slm_mul(speed, p->time_step); /* :125-127 */
    float sm, cm;
    slm_sincos(angle, &sm, &cm);
    x = slm_add(x, slm_mul(move_dist, cm));
    y = slm_add(y, slm_mul(move_dist, sm));

    float Wf = slm_i2f(W), Hf = slm_i2f(H); /* :130-133 */
    x = slm_fmod(x, Wf);
    if (x < 0.0f) x = slm_add(x, Wf);
    y = slm_fmod(y, Hf);
    if (y < 0.0f) y = slm_add(y, Hf);

    int64_t cell = -1; /* :136-141 */
    int32_t deposit_x = slm_f2i(x);
    int32_t deposit_y = slm_f2i(y);
    if (deposit_x >= 0 && deposit_x < W && deposit_y >= 0 && deposit_y < H)
        cell = (int64_t)deposit_y * W + deposit_x;

    a[0] = x; /* :144 */
    a[1] = y;
    a[2] = angle;
    a[3] = speed;
    return cell;
}

/* Sequential fold of k deposits: t <- clamp(t + dep, 0, 1), k times
 * (compute.wgsl:140 applied once per agent landing in the cell).  Once an
 * iteration leaves t's bits unchanged every later one does too. */
inline float fold_f32(float t, uint32_t k, float dep) {
    for (uint32_t i = 0; i < k; i++) {
        float nt = slm_clamp(slm_add(t, dep), 0.0f, 1.0f);
        if (slm_f2u_bits(nt) == slm_f2u_bits(t)) break;
        t = nt;
    }
    return t;
}

inline double fold_f64(double t, uint32_t k, double dep) {
    for (uint32_t i = 0; i < k; i++) {
        double v = t + dep;
        double nt = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
        if (nt == t) break;
        t = nt;
    }
    return t;
}

inline int64_t wrap_i(int64_t v, int64_t n) {
    v %= n;
    return v < 0 ? v + n : v;
}

int resolve_threads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

} // namespace

extern "C" {

/* One agent pass over AoS agents (x, y, angle, speed), reading `trail` and
 * adding 1 to counts[cell] for every deposit.  ids[i] (or i when ids is NULL)
 * is the agent_index that seeds the jitter hash.  With SLIME_DISPATCH_REFERENCE
 * an agent that the reference's dispatch visits m times (compute.wgsl:60,
 * src/main.rs:1174-1178; slm_dispatch_visits) is updated once from the state
 * the pass found and deposits m times; m = 0 leaves it untouched. */
void oracle_agents_pass(const SlimeParams* p, uint32_t W, uint32_t H, uint64_t n, float* agents,
                        const uint32_t* ids, const float* trail, uint32_t* counts, int threads) {
    int nt = resolve_threads(threads);
    const bool ref_dispatch = p->dispatch_mode == SLIME_DISPATCH_REFERENCE;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        int32_t index = ids ? (int32_t)ids[i] : (int32_t)i;
        uint32_t visits = ref_dispatch ? slm_dispatch_visits(n, (uint64_t)(uint32_t)index) : 1u;
        if (visits == 0) continue;
        int64_t cell = agent_update(p, (int32_t)W, (int32_t)H, index, agents + 4 * i, trail);
        if (cell >= 0) {
#pragma omp atomic
            counts[cell] += visits;
        }
    }
}

/* Deposit fold, decay_trail (compute.wgsl:148-161) and diffuse_trail
 * (compute.wgsl:164-195) from `trail` + `counts` into `out`. */
void oracle_trail_pass(const SlimeParams* p, uint32_t W, uint32_t H, const float* trail,
                       const uint32_t* counts, float* out, int threads) {
    int nt = resolve_threads(threads);
    const int64_t Wi = W, Hi = H, ncell = Wi * Hi;
    std::vector<float> d((size_t)ncell);
    const float dep = p->pheromone_deposition_amount;
    const float decay_k = slm_mul(p->decay_factor, 0.001f); /* :159 */
    const float rate = slm_clamp(p->diffusion_rate, 0.0f, 1.0f); /* :173 */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t c = 0; c < ncell; c++) {
        float v = fold_f32(trail[c], counts ? counts[c] : 0u, dep);
        if (p->decay_mode == SLIME_DECAY_MULTIPLY)
            v = slm_mul(v, p->decay_factor);
        else
            v = slm_max(slm_sub(v, decay_k), 0.0f); /* :160 */
        d[(size_t)c] = v;
    }
    if (p->blur_mode == SLIME_BLUR_GAUSS) {
        int R = slm_gauss_radius(p->blur_radius, SLIME_MAX_BLUR_RADIUS);
        float w[2 * SLIME_MAX_BLUR_RADIUS + 1];
        slm_gauss_weights(R, p->blur_sigma, w);
        std::vector<float> h((size_t)ncell);
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                float acc = 0.0f;
                for (int i = -R; i <= R; i++) acc = slm_fma(w[i + R], d[(size_t)(y * Wi + wrap_i(x + i, Wi))], acc);
                h[(size_t)(y * Wi + x)] = acc;
            }
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                float acc = 0.0f;
                for (int j = -R; j <= R; j++) acc = slm_fma(w[j + R], h[(size_t)(wrap_i(y + j, Hi) * Wi + x)], acc);
                out[y * Wi + x] = slm_mix(d[(size_t)(y * Wi + x)], acc, rate);
            }
    } else {
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                float sum = 0.0f; /* :176-189, dy outer, dx inner */
                for (int64_t dy = -1; dy <= 1; dy++)
                    for (int64_t dx = -1; dx <= 1; dx++) {
                        int64_t nx = (x + dx + Wi) % Wi;
                        int64_t ny = (y + dy + Hi) % Hi;
                        sum = slm_add(sum, d[(size_t)(ny * Wi + nx)]);
                    }
                float avg = slm_div(sum, 9.0f); /* :193 */
                out[y * Wi + x] = slm_mix(d[(size_t)(y * Wi + x)], avg, rate); /* :194 */
            }
    }
}

/* The same trail pass in binary64 (fold, decay and blur in double; Gaussian
 * weights unrounded). */
void oracle_trail_pass_f64(const SlimeParams* p, uint32_t W, uint32_t H, const double* trail,
                           const uint32_t* counts, double* out, int threads) {
    int nt = resolve_threads(threads);
    const int64_t Wi = W, Hi = H, ncell = Wi * Hi;
    std::vector<double> d((size_t)ncell);
    const double dep = p->pheromone_deposition_amount;
    const double decay = p->decay_factor;
    const double decay_k = decay * 0.001;
    double rate = p->diffusion_rate;
    rate = rate < 0.0 ? 0.0 : (rate > 1.0 ? 1.0 : rate);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t c = 0; c < ncell; c++) {
        double v = fold_f64(trail[c], counts ? counts[c] : 0u, dep);
        if (p->decay_mode == SLIME_DECAY_MULTIPLY)
            v = v * decay;
        else
            v = (v - decay_k) > 0.0 ? (v - decay_k) : 0.0;
        d[(size_t)c] = v;
    }
    if (p->blur_mode == SLIME_BLUR_GAUSS) {
        int R = slm_gauss_radius(p->blur_radius, SLIME_MAX_BLUR_RADIUS);
        double w[2 * SLIME_MAX_BLUR_RADIUS + 1], tot = 0.0;
        double s2 = 2.0 * (double)p->blur_sigma * (double)p->blur_sigma;
        for (int i = -R; i <= R; i++) tot += (w[i + R] = slm_exp_neg_host((double)(i * i) / s2));
        for (int i = 0; i <= 2 * R; i++) w[i] /= tot;
        std::vector<double> h((size_t)ncell);
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                double acc = 0.0;
                for (int i = -R; i <= R; i++) acc += w[i + R] * d[(size_t)(y * Wi + wrap_i(x + i, Wi))];
                h[(size_t)(y * Wi + x)] = acc;
            }
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                double acc = 0.0;
                for (int j = -R; j <= R; j++) acc += w[j + R] * h[(size_t)(wrap_i(y + j, Hi) * Wi + x)];
                double c = d[(size_t)(y * Wi + x)];
                out[y * Wi + x] = c * (1.0 - rate) + acc * rate;
            }
    } else {
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                double sum = 0.0;
                for (int64_t dy = -1; dy <= 1; dy++)
                    for (int64_t dx = -1; dx <= 1; dx++)
                        sum += d[(size_t)(((y + dy + Hi) % Hi) * Wi + (x + dx + Wi) % Wi)];
                double c = d[(size_t)(y * Wi + x)];
                out[y * Wi + x] = c * (1.0 - rate) + (sum / 9.0) * rate;
            }
    }
}

/* `steps` full steps in place over AoS agents and the trail.  counts_per_step,
 * when not NULL, receives the deposit counts of every step
 * (steps * W * H entries). */
void oracle_run(const SlimeParams* p, uint32_t W, uint32_t H, uint64_t n, float* agents, float* trail,
                uint32_t steps, uint32_t* counts_per_step, int threads) {
    const size_t ncell = (size_t)W * H;
    std::vector<uint32_t> counts(ncell);
    std::vector<float> next(ncell);
    for (uint32_t s = 0; s < steps; s++) {
        std::fill(counts.begin(), counts.end(), 0u);
        oracle_agents_pass(p, W, H, n, agents, nullptr, trail, counts.data(), threads);
        oracle_trail_pass(p, W, H, trail, counts.data(), next.data(), threads);
        memcpy(trail, next.data(), ncell * sizeof(float));
        if (counts_per_step) memcpy(counts_per_step + (size_t)s * ncell, counts.data(), ncell * sizeof(uint32_t));
    }
}

/* ---------------------------------------------------------------------------
 * Frozen-trajectory chain in binary64.  With the deposit counts k_s of every
 * step fixed, one step is T_{s+1} = Diffuse(Decay(Fold(T_s, k_s))), and the
 * loss is 0.5 * ||T_steps - target||^2.  The three trail-chain parameters are
 * passed as doubles so that finite differences can perturb them.
 */
struct ChainParams {
    uint32_t W, H, decay_mode, blur_mode;
    int R;
    double w[2 * SLIME_MAX_BLUR_RADIUS + 1];
    double decay, rate_raw, dep;
};

static void chain_setup(ChainParams* c, const SlimeParams* p, uint32_t W, uint32_t H, double decay,
                        double rate, double dep) {
    c->W = W;
    c->H = H;
    c->decay_mode = p->decay_mode;
    c->blur_mode = p->blur_mode;
    c->R = p->blur_mode == SLIME_BLUR_GAUSS ? slm_gauss_radius(p->blur_radius, SLIME_MAX_BLUR_RADIUS) : 1;
    if (p->blur_mode == SLIME_BLUR_GAUSS) {
        /* The binary32 weights the forward applies, evaluated in binary64:
         * the chain is the same linear operator the kernels implement. */
        float w32[2 * SLIME_MAX_BLUR_RADIUS + 1];
        slm_gauss_weights(c->R, p->blur_sigma, w32);
        for (int i = 0; i <= 2 * c->R; i++) c->w[i] = (double)w32[i];
    } else {
        for (int i = 0; i < 3; i++) c->w[i] = 1.0 / 3.0;
    }
    c->decay = decay;
    c->rate_raw = rate;
    c->dep = dep;
}

/* B(u): the (symmetric, toroidal) blur operator. */
static void chain_blur(const ChainParams* c, const double* u, double* out, double* tmp, int nt) {
    const int64_t Wi = c->W, Hi = c->H;
    const int R = c->R;
    if (c->blur_mode != SLIME_BLUR_GAUSS) {
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t y = 0; y < Hi; y++)
            for (int64_t x = 0; x < Wi; x++) {
                double s = 0.0;
                for (int64_t dy = -1; dy <= 1; dy++)
                    for (int64_t dx = -1; dx <= 1; dx++) s += u[wrap_i(y + dy, Hi) * Wi + wrap_i(x + dx, Wi)];
                out[y * Wi + x] = s / 9.0;
            }
        return;
    }
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t y = 0; y < Hi; y++)
        for (int64_t x = 0; x < Wi; x++) {
            double acc = 0.0;
            for (int i = -R; i <= R; i++) acc += c->w[i + R] * u[y * Wi + wrap_i(x + i, Wi)];
            tmp[y * Wi + x] = acc;
        }
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t y = 0; y < Hi; y++)
        for (int64_t x = 0; x < Wi; x++) {
            double acc = 0.0;
            for (int j = -R; j <= R; j++) acc += c->w[j + R] * tmp[wrap_i(y + j, Hi) * Wi + x];
            out[y * Wi + x] = acc;
        }
}

static inline double chain_rate(const ChainParams* c) {
    return c->rate_raw < 0.0 ? 0.0 : (c->rate_raw > 1.0 ? 1.0 : c->rate_raw);
}

static inline double chain_decay(const ChainParams* c, double f) {
    if (c->decay_mode == SLIME_DECAY_MULTIPLY) return f * c->decay;
    double v = f - c->decay * 0.001;
    return v > 0.0 ? v : 0.0;
}

/* Forward chain; returns the loss and writes T_steps to trail_final if not
 * NULL.  trails_all, if not NULL, receives T_0 .. T_steps ((steps+1)*W*H). */
static double chain_forward(const ChainParams* c, const double* trail0, const uint32_t* counts, uint32_t steps,
                            const double* target, double* trail_final, double* trails_all, int nt) {
    const size_t ncell = (size_t)c->W * c->H;
    std::vector<double> t(trail0, trail0 + ncell), u(ncell), b(ncell), tmp(ncell);
    const double r = chain_rate(c);
    if (trails_all) memcpy(trails_all, trail0, ncell * sizeof(double));
    for (uint32_t s = 0; s < steps; s++) {
        const uint32_t* k = counts + (size_t)s * ncell;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)ncell; i++) u[i] = chain_decay(c, fold_f64(t[i], k[i], c->dep));
        chain_blur(c, u.data(), b.data(), tmp.data(), nt);
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)ncell; i++) t[i] = u[i] * (1.0 - r) + b[i] * r;
        if (trails_all) memcpy(trails_all + (size_t)(s + 1) * ncell, t.data(), ncell * sizeof(double));
    }
    double loss = 0.0;
    if (target) {
#pragma omp parallel for schedule(static) reduction(+ : loss) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)ncell; i++) {
            double d = t[i] - target[i];
            loss += 0.5 * d * d;
        }
    }
    if (trail_final) memcpy(trail_final, t.data(), ncell * sizeof(double));
    return loss;
}

double oracle_chain_loss_f64(const SlimeParams* p, uint32_t W, uint32_t H, double decay, double rate,
                             double dep, const double* trail0, const uint32_t* counts, uint32_t steps,
                             const double* target, double* trail_final, int threads) {
    ChainParams c;
    chain_setup(&c, p, W, H, decay, rate, dep);
    return chain_forward(&c, trail0, counts, steps, target, trail_final, nullptr, resolve_threads(threads));
}

/* Hand-derived adjoint of the chain (the binary64 reference for the GPU
 * backward).  Writes dL/dT_0 to d_trail0 (if not NULL) and
 * grads[0..2] = dL/d(decay_factor), dL/d(diffusion_rate), dL/d(deposition).
 * The loss is 0.5*||T_steps - target||^2; alternatively pass target = NULL and
 * g_final = dL/dT_steps.  Conventions at kinks: a fold is differentiated as
 * unclamped iff k == 0 or 0 < Fold < 1; the subtractive decay is active iff
 * f - decay*0.001 > 0; the diffusion-rate clamp passes the gradient iff
 * 0 < rate < 1. */
static double chain_adjoint(const ChainParams& c, uint32_t W, uint32_t H, const std::vector<double>& trails,
                            double loss, const uint32_t* counts, uint32_t steps, const double* target,
                            const double* g_final, double* d_trail0, double* grads, int nt);

double oracle_chain_adjoint_f64(const SlimeParams* p, uint32_t W, uint32_t H, double decay, double rate,
                                double dep, const double* trail0, const uint32_t* counts, uint32_t steps,
                                const double* target, const double* g_final, double* d_trail0, double* grads,
                                int threads) {
    const int nt = resolve_threads(threads);
    ChainParams c;
    chain_setup(&c, p, W, H, decay, rate, dep);
    const size_t ncell = (size_t)W * H;
    std::vector<double> trails((size_t)(steps + 1) * ncell);
    double loss = chain_forward(&c, trail0, counts, steps, target, nullptr, trails.data(), nt);
    return chain_adjoint(c, W, H, trails, loss, counts, steps, target, g_final, d_trail0, grads, nt);
}

/* The same adjoint (binary64 arithmetic) along a given trajectory: the
 * trails T_0 .. T_steps of a binary32 forward (trails_f32, steps + 1 grids)
 * instead of the binary64 forward.  It separates the error of a binary32
 * backward's own arithmetic from the difference between the binary32 and
 * binary64 forwards it differentiates.  g_final = dL/dT_steps is required. */
double oracle_chain_adjoint_f64_along(const SlimeParams* p, uint32_t W, uint32_t H, double decay, double rate,
                                      double dep, const float* trails_f32, const uint32_t* counts, uint32_t steps,
                                      const double* g_final, double* d_trail0, double* grads, int threads) {
    const int nt = resolve_threads(threads);
    ChainParams c;
    chain_setup(&c, p, W, H, decay, rate, dep);
    const size_t n = (size_t)(steps + 1) * W * H;
    std::vector<double> trails(n);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; i++) trails[i] = (double)trails_f32[i];
    return chain_adjoint(c, W, H, trails, 0.0, counts, steps, nullptr, g_final, d_trail0, grads, nt);
}

static double chain_adjoint(const ChainParams& c, uint32_t W, uint32_t H, const std::vector<double>& trails,
                            double loss, const uint32_t* counts, uint32_t steps, const double* target,
                            const double* g_final, double* d_trail0, double* grads, int nt) {
    const size_t ncell = (size_t)W * H;
    std::vector<double> g(ncell), gu(ncell), f(ncell), u(ncell), bu(ncell), bg(ncell), tmp(ncell);
    const double* tf = trails.data() + (size_t)steps * ncell;
    for (size_t i = 0; i < ncell; i++) g[i] = target ? (tf[i] - target[i]) : g_final[i];
    const double r = chain_rate(&c);
    const bool rate_active = c.rate_raw > 0.0 && c.rate_raw < 1.0;
    double gd = 0.0, gr = 0.0, gp = 0.0;
    for (int64_t s = (int64_t)steps - 1; s >= 0; s--) {
        const double* ts = trails.data() + (size_t)s * ncell;
        const uint32_t* k = counts + (size_t)s * ncell;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)ncell; i++) {
            f[i] = fold_f64(ts[i], k[i], c.dep);
            u[i] = chain_decay(&c, f[i]);
        }
        chain_blur(&c, u.data(), bu.data(), tmp.data(), nt);
        chain_blur(&c, g.data(), bg.data(), tmp.data(), nt); /* B is symmetric: B^T = B */
        double sd = 0.0, sr = 0.0, sp = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : sd, sr, sp) num_threads(nt)
        for (int64_t i = 0; i < (int64_t)ncell; i++) {
            if (rate_active) sr += g[i] * (bu[i] - u[i]);
            double g_u = (1.0 - r) * g[i] + r * bg[i];
            double g_f;
            if (c.decay_mode == SLIME_DECAY_MULTIPLY) {
                sd += g_u * f[i];
                g_f = g_u * c.decay;
            } else {
                bool act = (f[i] - c.decay * 0.001) > 0.0;
                sd += act ? -0.001 * g_u : 0.0;
                g_f = act ? g_u : 0.0;
            }
            bool unclamped = k[i] == 0 || (f[i] > 0.0 && f[i] < 1.0);
            if (unclamped) sp += g_f * (double)k[i];
            gu[i] = unclamped ? g_f : 0.0;
        }
        gd += sd;
        gr += sr;
        gp += sp;
        g.swap(gu);
    }
    if (d_trail0) memcpy(d_trail0, g.data(), ncell * sizeof(double));
    grads[0] = gd;
    grads[1] = gr;
    grads[2] = gp;
    return loss;
}

/* The colourise pass of src/display.wgsl:44-86 on the host (headless): trail
 * -> LUT (R[256] G[256] B[256]) -> RGBA8, aspect-fit with black bars. */
void oracle_colorize(uint32_t W, uint32_t H, const float* trail, const uint8_t* lut, uint32_t tw, uint32_t th,
                     uint8_t* rgba) {
    float sim_w = (float)W, sim_h = (float)H, tex_w = (float)tw, tex_h = (float)th;
    float sim_aspect = slm_div(sim_w, sim_h), tex_aspect = slm_div(tex_w, tex_h);
    float scale, off_x = 0.0f, off_y = 0.0f;
    if (tex_aspect > sim_aspect) {
        scale = slm_div(tex_h, sim_h);
        off_x = slm_mul(slm_sub(tex_w, slm_mul(sim_w, scale)), 0.5f);
    } else {
        scale = slm_div(tex_w, sim_w);
        off_y = slm_mul(slm_sub(tex_h, slm_mul(sim_h, scale)), 0.5f);
    }
    for (uint32_t iy = 0; iy < th; iy++)
        for (uint32_t ix = 0; ix < tw; ix++) {
            float fx = slm_div(slm_sub((float)ix, off_x), scale);
            float fy = slm_div(slm_sub((float)iy, off_y), scale);
            uint8_t* o = rgba + 4 * ((size_t)iy * tw + ix);
            if (fx >= 0.0f && fx < sim_w && fy >= 0.0f && fy < sim_h) {
                int32_t x = slm_f2i(fx), y = slm_f2i(fy);
                float intensity = slm_clamp(trail[(size_t)y * W + x], 0.0f, 1.0f);
                uint32_t idx = (uint32_t)slm_f2i(slm_mul(intensity, 255.0f));
                o[0] = lut[idx];
                o[1] = lut[idx + 256];
                o[2] = lut[idx + 512];
                o[3] = 255;
            } else {
                o[0] = o[1] = o[2] = 0;
                o[3] = 255;
            }
        }
}

int oracle_num_threads(void) { return resolve_threads(0); }

/* The sensor samples (left, right, centre) of n agents, 3 floats each (the
 * tests pin them against the reference). */
void oracle_sense(const SlimeParams* p, uint32_t W, uint32_t H, uint64_t n, const float* agents, const float* trail,
                  float* out) {
    for (uint64_t i = 0; i < n; i++)
        sense(p, (int32_t)W, (int32_t)H, agents[4 * i], agents[4 * i + 1], agents[4 * i + 2], trail, &out[3 * i],
              &out[3 * i + 1], &out[3 * i + 2]);
}

/* slm_dispatch_visits(n, index[i]) for m indices. */
void oracle_dispatch_visits(uint64_t n, const uint64_t* index, uint64_t m, uint32_t* out) {
    for (uint64_t i = 0; i < m; i++) out[i] = slm_dispatch_visits(n, index[i]);
}

/* sample_trail_map at n positions (the tests pin it against the reference). */
void oracle_sample(const float* trail, uint32_t W, uint32_t H, const float* px, const float* py, uint64_t n,
                   float* out) {
    for (uint64_t i = 0; i < n; i++) out[i] = sample_trail_map(trail, (int32_t)W, (int32_t)H, px[i], py[i]);
}

/* The shared builtins, exported so the tests can check them. */
void oracle_sincos(const float* x, uint64_t n, float* s, float* c) {
    for (uint64_t i = 0; i < n; i++) slm_sincos(x[i], s + i, c + i);
}
void oracle_jitter_hash(const int32_t* index, const float* x, const float* y, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; i++) out[i] = slm_jitter_hash(index[i], x[i], y[i]);
}
void oracle_uniform01(uint64_t seed, uint64_t n, uint32_t field, float* out) {
    for (uint64_t i = 0; i < n; i++) out[i] = slm_uniform01(seed, i, field);
}
/* Number of binary32 inputs with biased exponent in [e_lo, e_hi] (both signs)
 * on which the fixed-window Payne-Hanek reduction differs from the table one
 * in the reduced argument's bits or the quadrant; e_lo >= 139, e_hi <= 170. */
uint64_t oracle_ph_window_mismatches(uint32_t e_lo, uint32_t e_hi) {
    if (e_lo < 139 || e_hi > 170 || e_lo > e_hi) return ~0ull;
    const int64_t per_sign = (int64_t)(e_hi - e_lo + 1) << 23;
    uint64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t i = 0; i < 2 * per_sign; i++) {
        uint32_t sign = i >= per_sign ? 1u : 0u;
        uint32_t rem = (uint32_t)(i - (sign ? per_sign : 0));
        uint32_t bits = (sign << 31) | ((e_lo + (rem >> 23)) << 23) | (rem & 0x7fffffu);
        float x = slm_u2f_bits(bits), r1, r2;
        int q1, q2;
        slm_reduce_pio2_ph(x, &r1, &q1);
        slm_reduce_pio2_win(x, &r2, &q2);
        bad += (slm_f2u_bits(r1) != slm_f2u_bits(r2) || q1 != q2) ? 1u : 0u;
    }
    return bad;
}
/* Number of binary32 inputs with biased exponent in [e_lo, e_hi] (both signs)
 * on which the 32-bit-word Payne-Hanek tail (slm_ph_finish) differs from its
 * 64-bit statement (slm_ph_finish_u64), both fed the table's window;
 * 139 <= e_lo <= e_hi <= 254. */
uint64_t oracle_ph_finish_mismatches(uint32_t e_lo, uint32_t e_hi) {
    if (e_lo < 139 || e_hi > 254 || e_lo > e_hi) return ~0ull;
    const int64_t per_sign = (int64_t)(e_hi - e_lo + 1) << 23;
    uint64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t i = 0; i < 2 * per_sign; i++) {
        uint32_t sign = i >= per_sign ? 1u : 0u;
        uint32_t rem = (uint32_t)(i - (sign ? per_sign : 0));
        uint32_t bits = (sign << 31) | ((e_lo + (rem >> 23)) << 23) | (rem & 0x7fffffu);
        uint32_t m, w[3];
        slm_ph_window_table(slm_u2f_bits(bits), &m, w);
        float r1, r2;
        int q1, q2;
        slm_ph_finish(m, w[0], w[1], w[2], sign, &r1, &q1);
        slm_ph_finish_u64(m, w[0], w[1], w[2], sign, &r2, &q2);
        bad += (slm_f2u_bits(r1) != slm_f2u_bits(r2) || q1 != q2) ? 1u : 0u;
    }
    return bad;
}
int oracle_gauss_weights(float radius, float sigma, float* w) {
    int R = slm_gauss_radius(radius, SLIME_MAX_BLUR_RADIUS);
    if (slm_gauss_weights(R, sigma, w) != 0) return -1;
    return R;
}

} /* extern "C" */
