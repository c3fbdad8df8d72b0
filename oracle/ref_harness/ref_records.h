// ref_records.h -- the plain records through which the harnesses of the
// reference's own code (ref_harness.cpp on the host, ref_gpu_harness.cu on
// the GPU) receive materials, the environment and the renderer settings.
// The layouts are the C ABI's (kittlespt_gb300/scenes.py MATERIAL_DTYPE,
// ENV_DTYPE, SETTINGS_DTYPE), so tests hand the same numpy records to the
// oracle, to these harnesses and to the library.
//
// TEST INFRASTRUCTURE ONLY.
#pragma once

struct MaterialRecord {
    float albedo[3]; float metallic, roughness, transmission, ior;
    float emission[3]; float emission_scale, normal_scale;
    int albedo_tex, orm_tex, transmission_tex, emission_tex, normal_tex, pad;
};
struct EnvRecord {
    float sun_angular_diameter, sun_phi, sun_theta, sun_emission_factor;
    float rayleigh[3]; float mie, mie_absorption, rayleigh_height, mie_height, pad;
};
struct SettingsRecord {
    int max_depth, bloom, karis, auto_exposure;
    float bloom_final_blend, bloom_internal_blend, frame_delta_ms, pad;
};
