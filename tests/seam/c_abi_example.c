/* A plain C (C99) caller of the library: one AO frame over a floor and a wall, through the
 * same calls a raw-native maintainer's bindings make (rn_init, rn_accel_build, rn_ao_frame,
 * rn_accel_free). Host buffers; the library stages them.
 *
 *   cc -std=c99 -I include tests/seam/c_abi_example.c -L raw-native_gb300 -lrn_ao -o ao_example
 *
 * Exit status: 0 after a frame, 3 when the library reports no usable device (the reference's
 * "unverifiable"), 1 on any other error. */
#include <stdio.h>
#include <stdlib.h>

#include "rn_ao.h"

enum { W = 64, H = 64 };

int main(void) {
    rn_status st;
    if (rn_ao_version() != RN_AO_ABI_VERSION) {
        fprintf(stderr, "ABI version %d, header %d\n", rn_ao_version(), RN_AO_ABI_VERSION);
        return 1;
    }
    int rc = rn_init(&st);
    if (rc == RN_ERR_NO_DEVICE) {
        printf("unverifiable: %s\n", st.message);
        return 3;
    }
    if (rc != RN_OK) {
        fprintf(stderr, "rn_init: %d %s\n", rc, st.message);
        return 1;
    }
    /* the floor y = 0 over [-1, 1]^2 and a wall at x = 0.5, one unit high: 4 triangles */
    static const float tris[4 * 9] = {
        -1, 0, -1,  1, 0, -1,  1, 0, 1,
        -1, 0, -1,  1, 0, 1,  -1, 0, 1,
        0.5f, 0, -1,  0.5f, 1, -1,  0.5f, 1, 1,
        0.5f, 0, -1,  0.5f, 1, 1,  0.5f, 0, 1,
    };
    rn_accel* accel = NULL;
    rc = rn_accel_build(tris, 4, 0, &accel, &st);
    if (rc != RN_OK) {
        fprintf(stderr, "rn_accel_build: %d %s\n", rc, st.message);
        return 1;
    }
    /* a G-buffer seen from straight above: every pixel covers the floor */
    static float pos[W * H * 3], nrm[W * H * 3], ao[W * H], sky[W * H], sun[W * H], ss[W * H], err[W * H];
    static uint8_t mask[W * H];
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const int i = y * W + x;
            pos[3 * i] = -1.0f + 2.0f * ((float)x + 0.5f) / W;
            pos[3 * i + 1] = 0.0f;
            pos[3 * i + 2] = -1.0f + 2.0f * ((float)y + 0.5f) / H;
            nrm[3 * i] = 0.0f;
            nrm[3 * i + 1] = 1.0f;
            nrm[3 * i + 2] = 0.0f;
            mask[i] = 1;
        }
    const rn_gbuf g = {W, H, pos, nrm, mask};
    const float to_light[3] = {0.0f, 1.0f, 0.0f};
    rn_reconcile_result res;
    rc = rn_ao_frame(&g, accel, 16, 0.5f, 24, 0.12f, to_light, RN_SKY, ao, sky, sun, ss, err, &res, &st);
    rn_accel_free(accel);
    if (rc != RN_OK) {
        fprintf(stderr, "rn_ao_frame: %d %s\n", rc, st.message);
        return 1;
    }
    float lo = 1.0f;
    for (int i = 0; i < W * H; ++i) lo = ao[i] < lo ? ao[i] : lo;
    printf("pixels %d rmse %.6f max_error %.6f verdict %s; lowest ray-traced AO %.4f\n", (int)res.pixels,
           res.rmse, res.max_error, res.within_tolerance ? "verified" : "refuted", lo);
    return 0;
}
