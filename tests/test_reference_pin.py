"""The oracle pinned against the reference itself.

src/compute.wgsl is translated mechanically to C++ (oracle/wgsl/translate.py;
WGSL types and builtins in oracle/wgsl/prelude.h) and built into oracle/_ref/
by oracle/build_oracle.py wherever the reference's source tree is present
(elsewhere these tests skip; the fixtures in tests/golden/wgsl/ carry the
pin to other machines).  The harness runs the shader's entry points
invocation by invocation, and the tests compare with the oracle bit for bit:

  * sample_trail_map at random, integer, edge, outside and NaN positions;
  * decay_trail over whole grids (an elementwise pass);
  * diffuse_trail, read Jacobi-style (the race-free reading of the in-place
    pass), alone and after decay_trail, against the oracle's fused pass;
  * `main`, the agent update, sensing the trail as the pass found it;
  * whole frames (agents, decay, diffuse) where the shader's deposits cannot
    race: deposition 1.0 on a trail in [0, 1], or cells one agent lands on.

WGSL leaves sin and cos to the implementation; both sides take them from
include/slime_math.h.  By default (SLIME_SENSOR_SHADER) the side sensors'
directions are cos/sin of the rounded angle -/+ a, as the shader writes
them, and everything compares bit for bit at every sensor angle, including
300 whole frames at the reference's default settings.  The opt-in rotated
mode (SLIME_SENSOR_ROTATED) forms them by rotating (cos angle, sin angle)
instead; it is compared agent by agent: it differs exactly where the few-ulp
difference in a sensor's position flips a turn decision.
"""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params
from wgsl import wgslref

if not wgslref.available():
    pytest.skip("the reference's source tree is not present", allow_module_level=True)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_bits(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    both_nan = np.isnan(a) & np.isnan(b)
    return np.array_equal(np.where(both_nan, 0, bits(a)), np.where(both_nan, 0, bits(b)))


def no_counts(W, H):
    return np.zeros((H, W), np.uint32)


def test_sampler_matches_reference():
    rng = np.random.default_rng(1)
    for W, H in ((97, 61), (2, 2), (4096, 3)):
        trail = rng.random((H, W), dtype=np.float32)
        n = 20000
        px = rng.uniform(-3, W + 3, n).astype(np.float32)
        py = rng.uniform(-3, H + 3, n).astype(np.float32)
        px[:200] = np.floor(px[:200])  # integer positions
        py[200:400] = np.float32(H - 1)  # last row: y1 = H is out of bounds
        px[400:600] = np.nextafter(np.float32(W - 1), np.float32(0))
        px[600] = np.nan
        py[601] = np.nan
        px[602] = -0.0
        px[603] = np.float32(-np.inf)
        py[604] = np.float32(-1e30)
        assert same_bits(oracle.sample(trail, px, py), wgslref.sample(trail, px, py)), (W, H)


def test_sampler_at_saturating_positions():
    """The one sampler difference, at positions of 2^31 cells and beyond:
    there i32(floor(p)) saturates to 2^31 - 1, x0 + 1 wraps to -2^31, the
    shader's bounds test passes and it reads outside the trail (WGSL makes
    that read implementation-defined).  The oracle (and the GPU) test
    x0 >= W - 1 instead, so such positions sample 0, as every other position
    off the grid does."""
    W, H = 97, 61
    trail = np.random.default_rng(9).random((H, W), dtype=np.float32) + np.float32(1)
    px = np.array([np.inf, 3e9, 5.0, 5.0], np.float32)
    py = np.array([5.0, 5.0, np.inf, 2.2e9], np.float32)
    assert np.all(oracle.sample(trail, px, py) == 0)
    got = wgslref.sample(trail, px, py)
    # The harness reads 0 outside the buffer.  At an infinite coordinate the
    # interpolation weight is infinite and mix(0, 0, inf) is NaN, which shows
    # the shader went past its bounds test (its early return gives 0).
    assert np.isnan(got[0]) and np.isnan(got[2])
    assert got[1] == 0 and got[3] == 0


@pytest.mark.parametrize("decay", [0.0, 10.0, 75.0, 1000.0])
def test_decay_matches_reference(decay):
    W, H = 83, 57
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=decay, diffusion_rate=0.0)
    trail = np.random.default_rng(2).uniform(-0.5, 1.5, (H, W)).astype(np.float32)
    assert same_bits(oracle.trail_pass(p, W, H, trail, no_counts(W, H)), wgslref.decay(p, trail))


@pytest.mark.parametrize("rate", [0.0, 0.3, 0.5, 1.0, 1.7, -0.2])
def test_diffuse_matches_reference(rate):
    W, H = 64, 45
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=0.0, diffusion_rate=rate)
    trail = np.random.default_rng(3).random((H, W), dtype=np.float32)
    assert same_bits(oracle.trail_pass(p, W, H, trail, no_counts(W, H)), wgslref.diffuse(p, trail))


@pytest.mark.parametrize("W,H", [(64, 45), (3, 3), (1, 5), (130, 2)])
def test_decay_then_diffuse_matches_the_fused_pass(W, H):
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=12.0, diffusion_rate=0.55)
    trail = np.random.default_rng(4).random((H, W), dtype=np.float32)
    ref = wgslref.diffuse(p, wgslref.decay(p, trail))
    assert same_bits(oracle.trail_pass(p, W, H, trail, no_counts(W, H)), ref)


def agent_cases(W, H, n, seed, huge_headings=True):
    a = agents_uniform(n, W, H, 30.0, 50.0, seed=seed)
    a[:64, 2] = np.float32(-7.0)  # negative headings
    if huge_headings:
        a[64:128, 2] = np.float32(1e6)
    a[128:192, 0] = np.nextafter(np.float32(W), np.float32(0))  # on the last column
    a[192:256, 3] = np.float32(500.0)  # speeds above the maximum
    return a


def test_agent_update_matches_reference_exactly_with_axis_sensors():
    """Sensor angle 0: both sensor modes coincide with the shader, so the
    whole update (speed clamp, sampling, turn, jitter hash, wrap, move) must
    agree bit for bit in either mode, huge headings included."""
    W, H, n = 256, 192, 40000
    trail = np.random.default_rng(5).random((H, W), dtype=np.float32)
    for mode in (0, 1):
        for jitter, turn in ((0.05, 0.3), (1.0, 0.43), (0.0, 2.0)):
            p = config0_params(W, H, agent_sensor_angle=0.0, agent_jitter=jitter, agent_turn_speed=turn,
                               pheromone_deposition_amount=0.0, agent_speed_min=30.0, agent_speed_max=50.0,
                               sensor_mode=mode)
            agents = agent_cases(W, H, n, seed=int(turn * 100))
            assert same_bits(oracle.sense(p, W, H, agents, trail), wgslref.sense(p, agents, trail))
            ref_a, _ = wgslref.agents_pass(p, agents, trail)
            got = agents.copy()
            oracle.agents_pass(p, W, H, got, trail)
            assert same_bits(got, ref_a), (mode, jitter, turn)


def pin_trail(kind, W, H, rng):
    if kind == "continuous":
        return rng.random((H, W), dtype=np.float32)
    return (rng.integers(0, 9, (H, W)) / 8.0).astype(np.float32)  # values 1/8 apart, many exact ties


@pytest.mark.parametrize("sensor_angle", [0.3, 0.4, 0.7854, 2.5])
@pytest.mark.parametrize("trail_kind", ["continuous", "eighths"])
def test_agent_update_matches_reference_exactly(sensor_angle, trail_kind):
    """The default sensor mode evaluates cos/sin(angle -/+ a) as the shader
    does: at the reference's sensor angle (0.3), config 0's (0.4), pi/4 and
    2.5 rad, on continuous and on tie-rich trails, with negative and huge
    initial headings, every sensor sample and every agent's whole update is
    the reference's bit for bit (no differing agent at all)."""
    W, H, n = 256, 192, 40000
    trail = pin_trail(trail_kind, W, H, np.random.default_rng(7))
    p = config0_params(W, H, agent_sensor_angle=sensor_angle, agent_jitter=0.05, agent_turn_speed=0.3,
                       pheromone_deposition_amount=0.0, agent_speed_min=30.0, agent_speed_max=50.0)
    assert p.sensor_mode == 0
    agents = agent_cases(W, H, n, seed=8)
    assert same_bits(oracle.sense(p, W, H, agents, trail), wgslref.sense(p, agents, trail))
    ref_a, _ = wgslref.agents_pass(p, agents, trail)
    got = agents.copy()
    oracle.agents_pass(p, W, H, got, trail)
    differ = ~np.all(bits(got) == bits(ref_a), axis=1)
    assert differ.sum() == 0, differ.sum()


def decision(s):
    """compute.wgsl:98-112: 0 straight on, 1 turn left, 2 turn right, 3 equal."""
    l, r, c = s[:, 0], s[:, 1], s[:, 2]
    return np.select([(c > l) & (c > r), l > r, r > l], [0, 1, 2], 3)


@pytest.mark.parametrize("sensor_angle", [0.4, 0.7854, 2.5])
@pytest.mark.parametrize("trail_kind", ["continuous", "eighths"])
def test_rotated_mode_differs_only_at_near_tie_turns(sensor_angle, trail_kind):
    """The opt-in rotated mode: the two evaluations of the side directions
    differ by a few ulp, so the sensor samples agree within 2 ulp(W) (trail
    values in [0, 1]) unless a sensor sits on the sampler's edge (0 on one
    side), and an agent's update differs from the reference's exactly when
    that difference flips its turn decision: every other agent, and every
    other part of the update, is bit for bit the reference's.  Measured: 4 to
    5 agents in 100,000 flip."""
    W, H, n = 256, 192, 40000
    trail = pin_trail(trail_kind, W, H, np.random.default_rng(7))
    p = config0_params(W, H, agent_sensor_angle=sensor_angle, agent_jitter=0.05, agent_turn_speed=0.3,
                       pheromone_deposition_amount=0.0, agent_speed_min=30.0, agent_speed_max=50.0,
                       sensor_mode=1)
    agents = agent_cases(W, H, n, seed=8, huge_headings=False)
    ours_s, ref_s = oracle.sense(p, W, H, agents, trail), wgslref.sense(p, agents, trail)
    # a sensor position x + d cos is rounded at ulp(x): a few-ulp change of
    # direction can move it by one ulp in x and y, a sample by 2 ulp(W)
    tol = 2 * np.spacing(np.float32(max(W, H))) + 1e-6
    close = np.abs(ours_s.astype(np.float64) - ref_s) <= tol
    # or one sensor sits on the bilinear sampler's edge (x0 = W - 1 or
    # y0 = H - 1 on one side only) and samples 0 there
    off_edge = (ours_s == 0) | (ref_s == 0)
    assert np.all(close | off_edge)
    assert (~close).sum() <= 10, (~close).sum()
    flipped = decision(ours_s) != decision(ref_s)
    ref_a, _ = wgslref.agents_pass(p, agents, trail)
    got = agents.copy()
    oracle.agents_pass(p, W, H, got, trail)
    differ = ~np.all(bits(got) == bits(ref_a), axis=1)
    assert np.array_equal(differ, flipped)
    assert differ.sum() <= n // 2000, differ.sum()


def test_sensor_samples_at_huge_headings():
    """Headings far outside [0, 2pi) (possible only in an initial state: every
    update wraps the heading into [0, 2pi)).  The default mode rounds
    angle -/+ a at the heading's ulp exactly as the shader does, so every
    sample is the reference's.  In the rotated mode the rotation is not
    rounded there (at 1e6, ulp = 0.0625 rad), so the side directions differ
    by up to ulp(heading) / 2 rad and a sensor 9 px out moves by up to
    9 ulp / 2 px; with trail values in [0, 1] a sample moves by at most that
    (outside [-pi, pi] WGSL gives cos and sin no accuracy at all).  The
    centre sensor is the same in both."""
    W, H, n = 256, 192, 20000
    trail = np.random.default_rng(10).random((H, W), dtype=np.float32)
    p = config0_params(W, H, pheromone_deposition_amount=0.0)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=12)
    agents[:, 2] = np.random.default_rng(13).uniform(-1e6, 1e6, n).astype(np.float32)
    assert same_bits(oracle.sense(p, W, H, agents, trail), wgslref.sense(p, agents, trail))
    p.sensor_mode = 1
    ours_s, ref_s = oracle.sense(p, W, H, agents, trail), wgslref.sense(p, agents, trail)
    assert same_bits(ours_s[:, 2], ref_s[:, 2])
    bound = 9.0 * np.spacing(np.abs(agents[:, 2])).astype(np.float64) / 2 + 2 * np.spacing(np.float32(W)) + 1e-6
    d = np.abs(ours_s[:, :2].astype(np.float64) - ref_s[:, :2])
    off_edge = (ours_s[:, :2] == 0) | (ref_s[:, :2] == 0)
    assert np.all((d <= bound[:, None]) | off_edge)


@pytest.mark.parametrize("W,H,sensor_angle", [(256, 192, 0.0), (97, 61, 0.0), (256, 192, 0.4), (97, 61, 0.7854)])
def test_full_steps_match_reference_at_saturating_deposition(W, H, sensor_angle):
    """Deposition 1.0 (the reference's default) on a trail in [0, 1]: every
    deposit leaves its cell at 1 whatever order the racing invocations take,
    so the reference's frame is deterministic.  25 whole frames, agents and
    trail, bit for bit, with axis sensors and at config 0's sensor angle."""
    n = 20000
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=0.97, diffusion_rate=0.5,
                       agent_sensor_angle=sensor_angle, pheromone_deposition_amount=1.0)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=14)
    trail = np.random.default_rng(15).random((H, W), dtype=np.float32)
    ref_a, ref_t = agents, trail
    for _ in range(25):
        ref_a, ref_t = wgslref.frame(p, ref_a, ref_t)
    got_a, got_t = agents.copy(), trail.copy()
    oracle.run(p, W, H, got_a, got_t, 25)
    assert same_bits(got_a, ref_a)
    assert same_bits(got_t, ref_t)
    # the deposits happened: without them the mean would stay near 0.48
    assert ref_t.mean() > 0.9


def test_one_pass_matches_reference_where_deposits_do_not_race():
    """Deposition 0.3: after one agent pass the trail equals the reference's
    on every cell that at most one agent lands on (where the shader's
    non-atomic update cannot lose a deposit)."""
    W, H, n = 256, 192, 30000
    p = config0_params(W, H, decay_mode=0, blur_mode=0, agent_sensor_angle=0.0,
                       pheromone_deposition_amount=0.3)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=16)
    trail = np.random.default_rng(17).random((H, W), dtype=np.float32)
    ref_a, ref_t = wgslref.agents_pass(p, agents, trail)
    got_a = agents.copy()
    counts = oracle.agents_pass(p, W, H, got_a, trail)
    assert same_bits(got_a, ref_a)
    fold_only = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=0.0, diffusion_rate=0.0,
                               pheromone_deposition_amount=0.3)
    folded = oracle.trail_pass(fold_only, W, H, trail, counts)
    single = counts <= 1
    assert same_bits(folded[single], ref_t[single])
    assert np.count_nonzero(counts == 1) > n // 2


@pytest.mark.parametrize("W,H,tw,th", [(97, 61, 1600, 900), (97, 61, 900, 1600), (64, 48, 64, 48), (64, 48, 128, 96),
                                       (300, 100, 301, 199), (5, 7, 33, 17), (1, 1, 3, 2)])
def test_display_colorize_matches_reference(W, H, tw, th):
    """display.wgsl's `main` (translated, one invocation per pixel) against
    the oracle's colourise: aspect fit with black bars, the trail clamped and
    mapped through the 768-entry LUT, stored as rgba8unorm."""
    rng = np.random.default_rng(W * 7 + tw)
    trail = rng.uniform(-0.2, 1.2, (H, W)).astype(np.float32)
    edge = np.array([0.0, 1.0, np.nextafter(np.float32(1), np.float32(0)), 0.5 / 255, 254.5 / 255, np.nan,
                     -0.0, 2.0 / 255], np.float32)
    trail.flat[:min(trail.size, edge.size)] = edge[:trail.size]
    lut = rng.integers(0, 256, 768, dtype=np.uint8)
    assert np.array_equal(oracle.colorize(W, H, trail, lut, tw, th), wgslref.colorize(trail, lut, tw, th))


def _radial_spectrum(t, nbins=24):
    f = np.abs(np.fft.fft2(t - t.mean())) ** 2
    ky = np.fft.fftfreq(t.shape[0])[:, None]
    kx = np.fft.fftfreq(t.shape[1])[None, :]
    bins = np.minimum((np.sqrt(kx ** 2 + ky ** 2) / 0.5 * nbins).astype(int), nbins - 1)
    return np.bincount(bins.ravel(), f.ravel(), nbins) / np.maximum(np.bincount(bins.ravel(), None, nbins), 1)


def _trail_stats(t):
    h, _ = np.histogram(t, bins=32, range=(0.0, 1.0))
    return float(t.astype(np.float64).sum()), h / h.sum(), _radial_spectrum(t.astype(np.float64))


def _stat_distance(a, b):
    """(relative trail-mass difference, histogram L1, largest |log ratio| of
    the radially averaged power spectra away from k = 0)."""
    return (abs(a[0] - b[0]) / b[0], float(np.abs(a[1] - b[1]).sum()),
            float(np.max(np.abs(np.log(a[2][1:] / b[2][1:])))))


def default_settings_params(W, H, **kw):
    """The reference's default settings (src/settings.rs:10-27) in its own
    decay and blur."""
    return config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, diffusion_rate=1.0,
                          agent_sensor_angle=0.3, agent_sensor_distance=20.0, agent_turn_speed=0.43, agent_jitter=0.0,
                          agent_speed_min=30.0, agent_speed_max=50.0, pheromone_deposition_amount=1.0, **kw)


def test_long_run_matches_reference_bit_for_bit():
    """300 frames at the reference's default settings (sensor angle 0.3,
    deposition 1.0, so the shader's frame is deterministic), 8,192 agents on
    128^2 from a zero trail: in the default sensor mode the oracle's run is
    the reference's, every agent and every trail cell of the last frame bit
    for bit, although the dynamics are chaotic (one flipped turn would make
    the runs part ways)."""
    W = H = 128
    n, frames = 8192, 300
    p = default_settings_params(W, H)
    ref_a, ref_t = agents_uniform(n, W, H, 30.0, 50.0, seed=1), np.zeros((H, W), np.float32)
    our_a, our_t = ref_a.copy(), ref_t.copy()
    for _ in range(frames):
        ref_a, ref_t = wgslref.frame(p, ref_a, ref_t)
    oracle.run(p, W, H, our_a, our_t, frames)
    assert same_bits(our_a, ref_a)
    assert same_bits(our_t, ref_t)
    assert ref_t.max() > 0.9  # deposits reached the trail (1.0, then one decay step)


def test_rotated_mode_long_run_statistics_match_reference():
    """The same 300 frames in the rotated sensor mode: its sensor directions
    flip a near-tie turn now and then and the dynamics are chaotic, so the
    two runs part ways (nearly every agent differs at the end).  Their trails
    must agree statistically: trail mass, value histogram and radial power
    spectrum are closer between the reference and the oracle from the same
    start than between the oracle and itself from three other random starts
    (measured: 0.026 / 0.036 / 0.25 against at least 0.091 / 0.086 / 0.68)."""
    W = H = 128
    n, frames = 8192, 300
    p = default_settings_params(W, H)
    ours_p = default_settings_params(W, H, sensor_mode=1)

    def ours(seed):
        a = agents_uniform(n, W, H, 30.0, 50.0, seed=seed)
        t = np.zeros((H, W), np.float32)
        oracle.run(ours_p, W, H, a, t, frames)
        return a, t

    ref_a, ref_t = agents_uniform(n, W, H, 30.0, 50.0, seed=1), np.zeros((H, W), np.float32)
    for _ in range(frames):
        ref_a, ref_t = wgslref.frame(p, ref_a, ref_t)
    our_a, our_t = ours(1)
    assert np.count_nonzero(~np.all(bits(ref_a) == bits(our_a), axis=1)) > n // 2  # the runs did part ways
    base = _trail_stats(our_t)
    to_ref = _stat_distance(_trail_stats(ref_t), base)
    seed_to_seed = [_stat_distance(_trail_stats(ours(s)[1]), base) for s in (2, 3, 4)]
    for k in range(3):
        assert to_ref[k] < min(d[k] for d in seed_to_seed), (k, to_ref, seed_to_seed)
