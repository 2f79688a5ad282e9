// A sphere, an upright cylinder and a capsule dropped on a fixed ground box,
// written against the C++ facade with the reference's geometry constructors
// (Geometry.h:16-18).  Exit code 0: all three at rest on the ground; 2: no CUDA
// device (expected on a machine without a GPU); 1: failed.
#include <cmath>
#include <cstdio>

#include "cpgpu_engine.hpp"

int main() {
    try {
        cpgpu::PhysicsEngine p;
        p.setStep_time(1.0 / 60.0);
        p.setSleepingEnabled(false);
        p.createRigidBody(cpgpu::ConvexUnionGeometry::box(cpgpu::Vec3(-50, -0.5, -50), 100, 0.5, 100), cpgpu::FIXED);
        cpgpu::RigidBody* s = p.createRigidBody(cpgpu::ConvexUnionGeometry::sphere(cpgpu::Vec3(-3, 3, 0), 0.5));
        cpgpu::RigidBody* c = p.createRigidBody(cpgpu::ConvexUnionGeometry::cylinder(cpgpu::Vec3(0, 3, 0), 0.5, 1.0));
        cpgpu::RigidBody* k = p.createRigidBody(cpgpu::ConvexUnionGeometry::capsule(cpgpu::Vec3(3, 3, 0), 0.3, 1.0));
        for (int i = 0; i < 400; i++) p.timeStep();
        bool ok = true;
        // rest heights of the centres of mass: sphere r, cylinder h/2, capsule
        // between lying (r) and standing (h/2 + r)
        const double lo[3] = {0.45, 0.45, 0.25}, hi[3] = {0.55, 0.55, 0.85};
        cpgpu::RigidBody* b[3] = {s, c, k};
        for (int i = 0; i < 3; i++) {
            cpgpu::Vec3 x = b[i]->getCOM(), v = b[i]->getVel();
            double speed = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
            std::printf("body %d y=%.4f |v|=%.3g\n", i, x.y, speed);
            ok = ok && x.y > lo[i] && x.y < hi[i] && speed < 5e-2;
        }
        return ok ? 0 : 1;
    } catch (const cpgpu::Error& e) {
        std::printf("%s\n", e.what());
        return e.code == CPGPU_ERR_NO_DEVICE ? 2 : 1;
    }
}
