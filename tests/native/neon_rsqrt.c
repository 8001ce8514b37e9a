/* Runs the Arm reciprocal-square-root estimate and step instructions the
 * reference's rsqrt_vec uses on aarch64 (vrsqrteq_f32, vrsqrtsq_f32) over
 * the inputs in argv[1] (raw float32) and writes est, step(x*est, est) and
 * the refined result to argv[2] (3 raw float32 per input). aarch64 only. */
#include <arm_neon.h>
#include <stdio.h>
#include <stdlib.h>

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* fi = fopen(argv[1], "rb");
    FILE* fo = fopen(argv[2], "wb");
    if (!fi || !fo) return 3;
    float in[4];
    size_t n;
    while ((n = fread(in, sizeof(float), 4, fi)) > 0) {
        for (size_t i = n; i < 4; ++i) in[i] = 1.0f;
        float32x4_t x = vld1q_f32(in);
        float32x4_t y0 = vrsqrteq_f32(x);
        float32x4_t s = vrsqrtsq_f32(vmulq_f32(x, y0), y0);
        float32x4_t y1 = vmulq_f32(y0, s);
        float e[4], st[4], r[4];
        vst1q_f32(e, y0);
        vst1q_f32(st, s);
        vst1q_f32(r, y1);
        for (size_t i = 0; i < n; ++i) {
            float o[3] = {e[i], st[i], r[i]};
            fwrite(o, sizeof(float), 3, fo);
        }
    }
    fclose(fi);
    fclose(fo);
    return 0;
}
