/* A plain C99 caller of the C ABI: a box dropped on a fixed ground box.
 * Exit code 0: it came to rest on the ground; 2: no CUDA device (expected on
 * a machine without a GPU, where every call must say so); 1: failed. */
#include <stdio.h>

#include "cpgpu.h"

int main(void) {
    cpgpu_world* w = NULL;
    int rc = cpgpu_world_create(&w);
    if (rc == CPGPU_ERR_NO_DEVICE) {
        printf("no CUDA device: %s\n", cpgpu_last_error());
        return 2;
    }
    if (rc != CPGPU_OK) return 1;
    const cpgpu_material m = {1.0, 0.3, 0.6, 1.1};
    const double ground[3] = {-50, -0.5, -50}, corner[3] = {0, 0, 0}, origin[3] = {0, 0, 0}, start[3] = {0, 3, 0};
    uint32_t g = 0, b = 0;
    if (cpgpu_body_box(w, ground, 100, 0.5, 100, &m, CPGPU_FIXED, origin, &g) != CPGPU_OK) return 1;
    if (cpgpu_body_box(w, corner, 1, 1, 1, &m, CPGPU_DYNAMIC, start, &b) != CPGPU_OK) return 1;
    if (cpgpu_step(w, 300) != CPGPU_OK) return 1;
    double com[6], quat[8], vel[6], ang[6];
    if (cpgpu_get_body_state(w, com, quat, vel, ang) != CPGPU_OK) return 1;
    printf("box y=%.4f vy=%.4g\n", com[4], vel[4]);
    cpgpu_world_destroy(w);
    return (com[4] > 0.45 && com[4] < 0.55) ? 0 : 1;
}
