// Box vs Ground (Demo/src/Demos/Tests/CollisionTests.h:77-165) written against
// the C++ facade exactly as the reference scenario is written against
// phyz::PhysicsEngine.  Exit code 0: passed; 2: no CUDA device (expected on a
// machine without a GPU); 1: failed.
#include <cmath>
#include <cstdio>

#include "cpgpu_engine.hpp"

int main() {
    try {
        cpgpu::PhysicsEngine p;
        p.setStep_time(1.0 / 60.0);
        p.setSleepingEnabled(false);
        cpgpu::ConvexUnionGeometry ground = cpgpu::ConvexUnionGeometry::box(cpgpu::Vec3(-50, -0.5, -50), 100, 0.5, 100);
        p.createRigidBody(ground, cpgpu::FIXED);
        cpgpu::RigidBody* box = p.createRigidBody(cpgpu::ConvexUnionGeometry::box(cpgpu::Vec3(0, 5, 0), 1, 1, 1));
        for (int i = 0; i < 300; i++) p.timeStep();
        cpgpu::Vec3 c = box->getCOM(), v = box->getVel();
        double speed = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        // a ray straight down onto the resting box hits its top face (y = 1) first
        cpgpu::RayHitInfo h = p.raycastFirstIntersection(cpgpu::Vec3(c.x, 10, c.z), cpgpu::Vec3(0, -1, 0));
        std::printf("box y=%.6f |v|=%.3g ray hit %d at %.4f\n", c.y, speed, h.did_hit ? (int)h.hit_object->getID() : 0,
                    h.hit_distance);
        bool ray_ok = h.did_hit && h.hit_object == box && std::fabs(h.hit_distance - (10 - (c.y + 0.5))) < 1e-3;
        return (std::fabs(c.y - 0.5) < 0.1 && speed < 5e-3 && ray_ok) ? 0 : 1;  // FP32 residual motion at rest
    } catch (const cpgpu::Error& e) {
        std::printf("%s\n", e.what());
        return e.code == CPGPU_ERR_NO_DEVICE ? 2 : 1;
    }
}
