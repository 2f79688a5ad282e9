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
        std::printf("box y=%.6f |v|=%.3g\n", c.y, speed);
        return (std::fabs(c.y - 0.5) < 0.1 && speed < 5e-3) ? 0 : 1;  // FP32 residual motion at rest
    } catch (const cpgpu::Error& e) {
        std::printf("%s\n", e.what());
        return e.code == CPGPU_ERR_NO_DEVICE ? 2 : 1;
    }
}
