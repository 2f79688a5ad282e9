// Bodies of several primitives built with ConvexUnionGeometry::merge and
// getTranslated (Geometry.h:34-37), written against the C++ facade: a table
// (a box top on four cylinder legs) dropped flat and an L of two boxes, on a
// fixed ground box.  Exit code 0: the table stands on its legs and both are at
// rest; 2: no CUDA device (expected on a machine without a GPU); 1: failed.
#include <cmath>
#include <cstdio>

#include "cpgpu_engine.hpp"

using cpgpu::ConvexUnionGeometry;
using cpgpu::Vec3;

int main() {
    try {
        cpgpu::PhysicsEngine p;
        p.setStep_time(1.0 / 60.0);
        p.setSleepingEnabled(false);
        p.createRigidBody(ConvexUnionGeometry::box(Vec3(-50, -0.5, -50), 100, 0.5, 100), cpgpu::FIXED);

        // table: top 2 x 0.2 x 2 at y in [1, 1.2], legs of radius 0.1 and height 1
        ConvexUnionGeometry table = ConvexUnionGeometry::box(Vec3(-1, 1, -1), 2, 0.2, 2);
        const double c[4][2] = {{-0.85, -0.85}, {0.85, -0.85}, {-0.85, 0.85}, {0.85, 0.85}};
        for (const auto& xz : c)
            table = ConvexUnionGeometry::merge(table, ConvexUnionGeometry::cylinder(Vec3(0, 0, 0), 0.1, 1.0)
                                                          .getTranslated(Vec3(xz[0], 0, xz[1])));
        cpgpu::RigidBody* t = p.createRigidBody(table.getTranslated(Vec3(-4, 0.5, 0)));

        ConvexUnionGeometry ell = ConvexUnionGeometry::merge(ConvexUnionGeometry::box(Vec3(0, 0, 0), 2, 0.5, 0.5),
                                                             ConvexUnionGeometry::box(Vec3(0, 0.5, 0), 0.5, 1.5, 0.5));
        cpgpu::RigidBody* l = p.createRigidBody(ell.getTranslated(Vec3(3, 1, 0)));

        for (int i = 0; i < 500; i++) p.timeStep();
        // the table's centre of mass: top 0.8 volume at y 1.1, legs 4 x 0.0314 at y 0.5
        const double table_y = (0.8 * 1.1 + 4 * M_PI * 0.01 * 0.5) / (0.8 + 4 * M_PI * 0.01);
        bool ok = true;
        cpgpu::RigidBody* b[2] = {t, l};
        const double lo[2] = {table_y - 0.03, 0.2}, hi[2] = {table_y + 0.03, 1.5};
        for (int i = 0; i < 2; i++) {
            Vec3 x = b[i]->getCOM(), v = b[i]->getVel();
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
