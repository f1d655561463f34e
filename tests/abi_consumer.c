/*
 * A C11 program that uses libsplatter_cuda.so through include/splatter.h alone, the way a compiled
 * host (the reference's Rust crate over extern "C", a C++ engine) would.  tests/test_abi_consumer.py
 * compiles it with -std=c11 -Wall -Wextra -Werror -pedantic (and the header once more as C++17) and
 * runs it:
 *
 *   abi_consumer host [file.ply]
 *       host-only entry points (no GPU): the viewer's default configuration, the uniform block,
 *       rejection of an invalid configuration, the identity motor, translator * rotor, a motor times
 *       its inverse, and, given a file, the validating header parser.  Prints "host ok".
 *   abi_consumer render W H FOVY DEPTH_SORTING COVARIANCE RECT OUT.rgba C0 .. C15
 *       Scene::new_dev_test (scene.rs:158-192) rendered once with SH order 0 and the UNORM8 blend;
 *       the RGBA8 image is written to OUT.rgba and the frame's counters are printed as
 *       "stats V DRAW N".
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "splatter.h"

#ifdef ABI_CONSUMER_RENDER
#include <cuda_runtime_api.h>
#endif

static int fail(const char* what, int rc) {
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, spl_last_error_string());
    return 1;
}

static int host_checks(const char* ply_path) {
    spl_config c;
    spl_renderer* r = NULL;
    unsigned char uniforms[224];
    const float cam[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0.25f, -0.5f, -5, 1};
    const float identity[8] = {1, 0, 0, 0, 0, 0, 0, 0};
    const float rotor[4] = {0.8f, 0.36f, 0.48f, 0.0f}, translation[3] = {0.5f, -1.0f, 2.0f};
    float motor[8], mat[16], inv[8], prod[8];
    int rc, k;

    spl_config_default(&c);
    if (c.radix_bits_per_digit != 8 || c.spherical_harmonics_order != 2 || c.depth_sorting != SPL_DEPTH_SORTING_GPU)
        return fail("spl_config_default (showcase.rs:39-50 literal)", -1);
    rc = spl_compute_uniforms(&c, cam, 64, 48, uniforms);
    if (rc != SPL_OK) return fail("spl_compute_uniforms", rc);
    c.radix_bits_per_digit = 3; /* does not divide 32 (renderer.rs:89-90) */
    rc = spl_renderer_create(&c, &r);
    if (rc != SPL_ERR_INVALID || r != NULL) return fail("spl_renderer_create accepted radix_bits_per_digit 3", rc);

    rc = spl_motor_to_mat4(identity, mat);
    if (rc != SPL_OK) return fail("spl_motor_to_mat4", rc);
    for (k = 0; k < 16; ++k)
        if (mat[k] != (k % 5 == 0 ? 1.0f : 0.0f)) return fail("identity motor -> identity matrix", k);
    rc = spl_motor_from_rotor_translation(rotor, translation, motor);
    if (rc != SPL_OK) return fail("spl_motor_from_rotor_translation", rc);
    rc = spl_motor_to_mat4(motor, mat);
    if (rc != SPL_OK) return fail("spl_motor_to_mat4", rc);
    for (k = 0; k < 3; ++k) { /* the origin's image (fourth column) is the translation */
        const float d = mat[12 + k] - translation[k];
        if (d > 1e-5f || d < -1e-5f) return fail("translator * rotor moves the origin by t", k);
    }
    rc = spl_motor_inverse(motor, inv);
    if (rc == SPL_OK) rc = spl_motor_product(motor, inv, prod);
    if (rc != SPL_OK) return fail("spl_motor_inverse / spl_motor_product", rc);
    for (k = 0; k < 8; ++k) {
        const float want = k == 0 ? 1.0f : 0.0f, d = prod[k] - want;
        if (d > 1e-5f || d < -1e-5f) return fail("motor * inverse(motor) == 1", k);
    }

    if (ply_path) {
        uint32_t header_bytes = 0;
        uint64_t count = 0;
        rc = spl_validate_file_header(ply_path, 1, &header_bytes, &count);
        if (rc != SPL_OK) return fail("spl_validate_file_header", rc);
        printf("header %u %llu\n", (unsigned)header_bytes, (unsigned long long)count);
    }
    printf("host ok\n");
    return 0;
}

#ifdef ABI_CONSUMER_RENDER
static int render(int argc, char** argv) {
    spl_config c;
    spl_renderer* r = NULL;
    spl_scene* s = NULL;
    spl_frame_info info;
    float cam[16];
    void* dev = NULL;
    unsigned char* host = NULL;
    uint32_t w, h;
    size_t bytes;
    FILE* f;
    int rc, k;

    if (argc != 25) {
        fprintf(stderr, "render: W H FOVY DEPTH_SORTING COVARIANCE RECT OUT.rgba and 16 camera floats\n");
        return 2;
    }
    w = (uint32_t)strtoul(argv[2], NULL, 10);
    h = (uint32_t)strtoul(argv[3], NULL, 10);
    spl_config_default(&c);
    c.field_of_view_y = strtof(argv[4], NULL);
    c.depth_sorting = (int32_t)strtol(argv[5], NULL, 10);
    c.use_covariance_for_scale = (int32_t)strtol(argv[6], NULL, 10);
    c.use_unaligned_rectangles = (int32_t)strtol(argv[7], NULL, 10);
    c.spherical_harmonics_order = 0;
    c.max_splat_count = 16;
    c.blend_mode = SPL_BLEND_UNORM8;
    for (k = 0; k < 16; ++k) cam[k] = strtof(argv[9 + k], NULL);
    bytes = (size_t)w * h * 4;

    rc = spl_renderer_create(&c, &r);
    if (rc != SPL_OK) return fail("spl_renderer_create", rc);
    rc = spl_scene_create_dev_test(r, &s);
    if (rc != SPL_OK) return fail("spl_scene_create_dev_test", rc);
    if (cudaMalloc(&dev, bytes) != cudaSuccess) return fail("cudaMalloc", -1);
    rc = spl_render_frame(r, s, cam, w, h, dev, NULL);
    if (rc != SPL_OK) return fail("spl_render_frame", rc);
    rc = spl_renderer_frame_info(r, &info); /* waits for the frame */
    if (rc != SPL_OK) return fail("spl_renderer_frame_info", rc);
    host = (unsigned char*)malloc(bytes);
    if (!host || cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return fail("readback", -1);
    f = fopen(argv[8], "wb");
    if (!f || fwrite(host, 1, bytes, f) != bytes) return fail("write", -1);
    fclose(f);
    printf("stats %llu %llu %llu\n", (unsigned long long)info.visible_count, (unsigned long long)info.draw_count,
           (unsigned long long)info.splat_count);
    free(host);
    cudaFree(dev);
    spl_scene_destroy(s);
    spl_renderer_destroy(r);
    return 0;
}
#endif

int main(int argc, char** argv) {
    if (argc >= 2 && strcmp(argv[1], "host") == 0) return host_checks(argc >= 3 ? argv[2] : NULL);
#ifdef ABI_CONSUMER_RENDER
    if (argc >= 2 && strcmp(argv[1], "render") == 0) return render(argc, argv);
#endif
    fprintf(stderr, "usage: abi_consumer host [file.ply] | render ...\n");
    return 2;
}
