"""The C ABI library: builds, loads, exports every declared symbol, and its
host-only entry points (settings, presets, parameter translation, error
paths) behave like the reference's Settings/presets (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in ("slime.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(slime_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built_lib):
    from slime_gb300 import _abi
    declared = declared_functions()
    assert len(declared) > 40
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(slime_[a-z0-9_]+)\b", out))
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    assert declared <= set(_abi.SIGNATURES), sorted(declared - set(_abi.SIGNATURES))


def test_struct_layouts():
    from slime_gb300 import SlimeParams, SlimeSettings, SlimeOptions, SlimeGrads
    # SimSizeUniform is 14 x 4 bytes (src/main.rs:29-46); the extensions add 24.
    assert C.sizeof(SlimeParams) == 80
    assert SlimeParams.blur_sigma.offset == 48 and SlimeParams._pad.offset == 52
    assert SlimeParams.time_step.offset == 56
    assert SlimeParams.dispatch_mode.offset == 68 and SlimeParams.sensor_mode.offset == 72
    assert C.sizeof(SlimeGrads) == 32
    assert C.sizeof(SlimeOptions) == 32


def test_settings_default_matches_reference(built_lib):
    import slime_gb300 as sg
    s = sg.default_settings()
    # src/settings.rs:4-27
    assert s.agent_count == 10_000_000
    assert (s.window_width, s.window_height, s.window_fullscreen) == (1600, 900, 0)
    assert s.agent_speed_min == 30.0 and s.agent_speed_max == 50.0
    assert s.agent_turn_speed == pytest.approx(0.43)
    assert s.agent_sensor_angle == pytest.approx(0.3) and s.agent_sensor_distance == 20.0
    assert s.pheromone_decay_factor == 10.0 and s.pheromone_diffusion_rate == 1.0
    assert s.pheromone_deposition_amount == 1.0 and s.agent_jitter == 0.0
    assert s.blur_radius == 2.0 and s.blur_sigma == 1.0
    assert (s.agent_possible_starting_headings_start, s.agent_possible_starting_headings_end) == (0.0, 360.0)


def test_presets_match_reference(built_lib):
    import slime_gb300 as sg
    names = sg.preset_names()
    assert names == ["Default", "Sponge", "Firecracker Trees", "Threads", "Curls", "Waves", "Snake", "Mesh"]
    curls = sg.preset("Curls")  # src/presets.rs:93-107
    assert curls.agent_count == 3_000_000 and curls.agent_jitter == 5.0
    assert curls.pheromone_decay_factor == 75.0 and curls.pheromone_diffusion_rate == pytest.approx(0.1)
    mesh = sg.preset("Mesh")  # src/presets.rs:139-152
    assert mesh.agent_sensor_distance == 225.0 and mesh.agent_sensor_angle == pytest.approx(1.57)
    assert mesh.agent_turn_speed == 6.0 and mesh.agent_count == 10_000_000
    with pytest.raises(KeyError):
        sg.preset("Nope")


def test_params_from_settings_is_sim_size_uniform_new(built_lib):
    import slime_gb300 as sg
    s = sg.preset("Snake")
    p = sg.params_from_settings(s, 1600, 900)
    assert (p.width, p.height) == (1600, 900)
    assert p.decay_factor == s.pheromone_decay_factor
    assert p.diffusion_rate == s.pheromone_diffusion_rate
    assert p.pheromone_deposition_amount == s.pheromone_deposition_amount
    assert p.agent_sensor_distance == 225.0 and p.blur_radius == 2.0 and p.blur_sigma == 1.0
    assert p.time_step == pytest.approx(0.016) and p.decay_mode == 0 and p.blur_mode == 0


def test_create_without_gpu_reports_no_device(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import slime_gb300 as sg
    with pytest.raises(sg.SlimeError) as e:
        sg.Simulation(16, 16, 4)
    assert e.value.status == -6


def test_invalid_sizes_rejected_before_touching_the_device(built_lib):
    import slime_gb300 as sg
    L = sg.lib()
    st = C.c_int(0)
    assert not L.slime_create(0, 16, 4, C.byref(st)) and st.value == -1
    assert not L.slime_create(65536, 65536, 4, C.byref(st)) and st.value == -1
    assert not L.slime_create(16, 16, 1 << 31, C.byref(st)) and st.value == -1
    assert L.slime_status_string(-5) == b"device-side wait timed out"


def test_package_refuses_to_run_without_its_library(tmp_path):
    """No CPU fallback: a package whose library is absent raises on first use."""
    import slime_gb300._abi as abi
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        abi.load(str(tmp_path / "libslime_gb300.so"))


def test_host_destinations_are_checked_before_the_library_writes():
    """The C calls write a fixed number of elements into the caller's
    buffer; the Python mirror refuses a destination of the wrong size, type
    or layout, and a gradient of the wrong size, before any call."""
    import numpy as np

    import slime_gb300 as sg
    sim = object.__new__(sg.Simulation)  # no device needed: nothing reaches the library
    sim._L, sim._h, sim._inflight = None, None, {}
    sim.width, sim.height, sim.n_agents = 8, 4, 3
    bad_trails = [np.empty((4, 7), np.float32), np.empty((4, 8), np.float64),
                  np.empty((8, 8), np.float32)[:, ::2], np.empty(32, np.int32)]
    for out in bad_trails:
        with pytest.raises(ValueError):
            sim.download_trail(out)
        with pytest.raises(ValueError):
            sim.download_trail_async(out)
    for out in (np.empty((2, 4), np.float32), np.empty((3, 4), np.float16), np.empty((3, 4), np.float32).T):
        with pytest.raises(ValueError):
            sim.download_agents(out)
    ro = np.empty((4, 8), np.float32)
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        sim.download_trail(ro)
    with pytest.raises(ValueError):
        sim.backward(np.zeros(31, np.float32))
    lut = np.zeros(768, np.uint8)
    for out in (np.empty((4, 8, 3), np.uint8), np.empty((4, 8, 4), np.float32), np.empty((4, 8), np.uint8)):
        with pytest.raises(ValueError):
            sim.colorize_async(lut, out)
    with pytest.raises(ValueError):
        sg.Ensemble([64, 64], [64], [10, 10], [None, None])


C_TO_RUST = {
    "uint32_t": "u32", "uint64_t": "u64", "int": "c_int", "float": "f32", "double": "f64", "size_t": "usize",
    "uint8_t": "u8", "char": "c_char", "void": "c_void",
}


def c_type_to_rust(t):
    """A C parameter or return type of include/slime.h in the Rust binding's
    spelling: `const float*` -> `*const f32`, `void**` -> `*mut *mut c_void`,
    `const char**` -> `*mut *const c_char`, `slime_ctx*` -> `*mut slime_ctx`."""
    t = " ".join(t.replace("*", " * ").split())
    stars = t.count("*")
    base = t.replace("*", "").split()
    const = base[0] == "const"
    name = base[-1]
    rust = C_TO_RUST.get(name, name)
    if stars == 0:
        return rust
    inner = ("*const " if const else "*mut ") + rust
    return "*mut " * (stars - 1) + inner


def header_declarations():
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "slime.h")).read(), flags=re.S)
    decls = {}
    for m in re.finditer(r"^([\w\s\*]+?)\b(slime_\w+)\s*\(([^;{]*?)\)\s*;", src, re.M):
        ret = c_type_to_rust(m.group(1).strip())
        args = []
        for a in m.group(3).split(","):
            a = " ".join(a.split())
            if not a or a == "void":
                continue
            ty = re.sub(r"\s*\b\w+$", "", a)  # drop the parameter name
            args.append(c_type_to_rust(ty))
        decls[m.group(2)] = (args, None if ret == "c_void" else ret)
    return decls, src


def rust_source():
    return open(os.path.join(ROOT, "rust", "slime_cuda", "src", "lib.rs")).read()


def test_rust_binding_declares_every_entry_point_with_the_header_types():
    """rust/slime_cuda/src/lib.rs (not compiled here: no Rust toolchain in
    this image) declares every function of include/slime.h with the same
    argument and return types, and nothing else."""
    decls, _ = header_declarations()
    src = rust_source()
    block = src[src.index('unsafe extern "C" {'):]
    block = block[:block.index("\n    }\n")]
    bound = {}
    for m in re.finditer(r"pub fn (slime_\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, re.S):
        args = [" ".join(a.split(":", 1)[1].split()) for a in m.group(2).split(",") if a.strip()]
        ret = " ".join(m.group(3).split()) if m.group(3) else None
        bound[m.group(1)] = (args, ret)
    assert set(bound) == set(decls), (sorted(set(decls) - set(bound)), sorted(set(bound) - set(decls)))
    for name, (args, ret) in decls.items():
        assert bound[name] == (args, ret), (name, bound[name], (args, ret))


def test_rust_binding_structs_and_constants_match_the_header():
    _, src_h = header_declarations()
    src_r = rust_source()
    structs = re.findall(r"typedef struct (\w+) \{(.*?)\} \1;", src_h, re.S)
    assert len(structs) == 6
    for name, body in structs:
        c_fields = []
        for line in body.split(";"):
            line = " ".join(line.split())
            if line:
                ty, field = line.rsplit(" ", 1)
                c_fields.append((field, c_type_to_rust(ty)))
        m = re.search(r"pub struct %s \{(.*?)\n    \}" % name, src_r, re.S)
        assert m, name
        r_fields = [tuple(x.strip() for x in f.split(":")) for f in re.findall(r"pub (\w+: \w+),", m.group(1))]
        r_fields = [(f, t) for f, t in r_fields]
        assert r_fields == c_fields, name
        assert "#[repr(C)]" in src_r[:m.start()].rsplit("pub struct", 1)[-1] or \
            src_r[:m.start()].rstrip().endswith(")]")
    defines = dict(re.findall(r"#define (SLIME_\w+) \(?(-?\d+)u?\)?", src_h))
    consts = dict(re.findall(r"pub const (SLIME_\w+): \w+ = (-?\d+);", src_r))
    assert defines == consts
