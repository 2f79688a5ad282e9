// shapes.cuh — device-side world-frame geometry of the body kinds (convex
// hull, sphere, cylinder, capsule, static triangle mesh) shared by the
// pose/AABB kernels.
#pragma once
#include "devmath.cuh"
#include "layout.h"

namespace cpgpu {

__device__ __forceinline__ void aabb_add(f3 p, f3* mn, f3* mx) {
    mn->x = fminf(mn->x, p.x); mn->y = fminf(mn->y, p.y); mn->z = fminf(mn->z, p.z);
    mx->x = fmaxf(mx->x, p.x); mx->y = fmaxf(mx->y, p.y); mx->z = fmaxf(mx->z, p.z);
}

// gen_AABB of the body's primitive at pose (com c, rotation R):
// Polyhedron::gen_AABB (ConvexPrimitive.cpp:660-676) over the world vertices,
// Sphere::gen_AABB (:439-443) centre +- radius, Cylinder::gen_AABB (:289-298)
// over both cap 8-gons, the bottom one re-derived as top - height * axis
// (Cylinder::recomputeFromReference, :272-287).
__device__ __forceinline__ void shape_aabb(const uint8_t* blob, f3 c, const M33& R, f3* mn, f3* mx) {
    const HullHeader* H = reinterpret_cast<const HullHeader*>(blob);
    if (H->kind == SHAPE_MESH) {   // StaticMeshGeometry: world-space triangles
        *mn = mk(*reinterpret_cast<const float4*>(blob + sizeof(HullHeader)));
        *mx = mk(*reinterpret_cast<const float4*>(blob + sizeof(HullHeader) + 16));
        return;
    }
    *mn = mk(INFINITY, INFINITY, INFINITY);
    *mx = mk(-INFINITY, -INFINITY, -INFINITY);
    if (H->kind == SHAPE_SPHERE) {
        float4 s = *reinterpret_cast<const float4*>(blob + sizeof(HullHeader));
        f3 w = c + mul(R, mk(s));
        *mn = w - mk(s.w, s.w, s.w);
        *mx = w + mk(s.w, s.w, s.w);
        return;
    }
    if (H->kind == SHAPE_CAPSULE) {
        // Capsule::gen_AABB (ConvexPrimitive.cpp:390-401): centre +- (|axis h/2| + r)
        float4 s = *reinterpret_cast<const float4*>(blob + sizeof(HullHeader));
        float4 ax = *reinterpret_cast<const float4*>(blob + kCylOffAxis);
        f3 w = c + mul(R, mk(s));
        f3 v = mul(R, mk(ax)) * (0.5f * ax.w);
        f3 e = mk(fabsf(v.x) + s.w, fabsf(v.y) + s.w, fabsf(v.z) + s.w);
        *mn = w - e;
        *mx = w + e;
        return;
    }
    if (H->kind == SHAPE_CYLINDER) {
        float4 ax = *reinterpret_cast<const float4*>(blob + kCylOffAxis);
        f3 axw = mul(R, mk(ax));
        const float4* top = reinterpret_cast<const float4*>(blob + kCylOffTop);
        for (int k = 0; k < kCylCap; k++) {
            f3 t = mul(R, mk(top[k])) + c;
            aabb_add(t, mn, mx);
            aabb_add(t - ax.w * axw, mn, mx);
        }
        return;
    }
    const float4* v = reinterpret_cast<const float4*>(blob + sizeof(HullHeader));
    for (int k = 0; k < H->nv; k++) aabb_add(c + mul(R, mk(v[k])), mn, mx);
}

}  // namespace cpgpu
