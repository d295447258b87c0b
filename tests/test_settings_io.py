"""Settings as a parameter file (slime_settings_to_text / _from_text /
_save / _load): every field of Settings (src/settings.rs:30-47) round-trips
exactly for the default settings and all eight presets (src/presets.rs:45-155),
the text is TOML that a standard parser reads back to the same values, and
malformed input is refused with the offending line."""
import math

import numpy as np
import pytest


FIELDS = ["agent_count", "agent_jitter", "agent_possible_starting_headings_start",
          "agent_possible_starting_headings_end", "agent_speed_max", "agent_speed_min", "agent_turn_speed",
          "pheromone_decay_factor", "pheromone_diffusion_rate", "pheromone_deposition_amount", "window_fullscreen",
          "window_height", "window_width", "agent_sensor_angle", "agent_sensor_distance", "blur_radius",
          "blur_sigma"]


def same(a, b):
    return bytes(a) == bytes(b)


def all_settings():
    import slime_gb300 as sg
    out = [("default", sg.default_settings())]
    out += [(name, sg.preset(name)) for name in sg.preset_names()]
    return out


def test_every_preset_round_trips_through_text_and_files(built_lib, tmp_path):
    import slime_gb300 as sg
    cases = all_settings()
    assert len(cases) == 9
    for name, s in cases:
        text = sg.settings_to_text(s)
        assert same(sg.settings_from_text(text), s), name
        path = tmp_path / f"{name}.toml"
        sg.save_settings(s, path)
        assert path.read_text() == text
        assert same(sg.load_settings(path), s), name


def test_text_is_toml_with_the_reference_field_names(built_lib):
    tomllib = pytest.importorskip("tomllib")
    import slime_gb300 as sg
    for name, s in all_settings():
        d = tomllib.loads(sg.settings_to_text(s))
        heads = d.pop("agent_possible_starting_headings")
        assert np.float32(heads["start"]) == np.float32(s.agent_possible_starting_headings_start)
        assert np.float32(heads["end"]) == np.float32(s.agent_possible_starting_headings_end)
        assert d["window_fullscreen"] is bool(s.window_fullscreen)
        for k in FIELDS:
            if k.startswith("agent_possible") or k == "window_fullscreen":
                continue
            got = d[k]
            if isinstance(got, float):
                assert np.float32(got) == np.float32(getattr(s, k)), (name, k)
            else:
                assert got == getattr(s, k), (name, k)


def test_binary32_values_round_trip_exactly(built_lib):
    import slime_gb300 as sg
    rng = np.random.default_rng(3)
    for _ in range(200):
        s = sg.default_settings()
        for k in FIELDS:
            if isinstance(getattr(s, k), float):
                v = np.float32(rng.choice([rng.uniform(-1e3, 1e3), rng.uniform(-1e-30, 1e-30),
                                           rng.uniform(-3e38, 3e38), 0.1, 1 / 3]))
                setattr(s, k, float(v))
        s.agent_count = int(rng.integers(0, 2 ** 63))
        s.window_width = int(rng.integers(0, 2 ** 32))
        s.window_fullscreen = int(rng.integers(0, 2))
        assert same(sg.settings_from_text(sg.settings_to_text(s)), s)
    s = sg.default_settings()
    s.agent_jitter, s.blur_sigma, s.blur_radius = math.inf, -math.inf, -0.0
    back = sg.settings_from_text(sg.settings_to_text(s))
    assert same(back, s)
    s.agent_jitter = math.nan
    assert math.isnan(sg.settings_from_text(sg.settings_to_text(s)).agent_jitter)


def test_partial_text_starts_from_the_defaults(built_lib):
    import slime_gb300 as sg
    s = sg.settings_from_text("# only two keys\n\nagent_count = 1_000  # comment\nagent_sensor_angle = 0.4\n")
    d = sg.default_settings()
    assert s.agent_count == 1000 and np.float32(s.agent_sensor_angle) == np.float32(0.4)
    s.agent_count, s.agent_sensor_angle = d.agent_count, d.agent_sensor_angle
    assert same(s, d)


@pytest.mark.parametrize("text,line", [
    ("agent_count = 1\nno_such_key = 2\n", 2),
    ("agent_count = -5\n", 1),
    ("window_width = 4294967296\n", 1),
    ("agent_jitter = 0.1x\n", 1),
    ("window_fullscreen = yes\n", 1),
    ("agent_jitter = 1\nagent_jitter = 2\n", 2),
    ("\n\nagent_possible_starting_headings = { start = 0.0 }\n", 3),
    ("agent_count\n", 1),
])
def test_malformed_text_is_refused_with_its_line(built_lib, text, line):
    import slime_gb300 as sg
    with pytest.raises(ValueError, match=f"bad line {line}"):
        sg.settings_from_text(text)


def test_missing_file_is_an_error(built_lib, tmp_path):
    import slime_gb300 as sg
    with pytest.raises(ValueError):
        sg.load_settings(tmp_path / "absent.toml")
