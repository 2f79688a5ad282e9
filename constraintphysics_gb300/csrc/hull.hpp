// hull.hpp — host-side preparation of convex hull shapes for the device path.
//
// Mirrors what Polyhedron::Polyhedron (ConstraintPhysics/src/ConvexPrimitive.cpp:
// 582-658) derives from (points, faces): face normals with the reference's
// normal/winding rule, the edge list, vertex adjacency and the Gauss map with
// cached face extrema and antipodal-redundancy flags (:861-896).  Feature ids
// (vertex, surface = n_points + face, edge ids of clipped points) depend on
// these orders, so they are reproduced exactly; the arithmetic is FP64 here and
// the packed blob the device reads is FP32.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>

namespace cpgpu {

struct D3 {
    double x = 0, y = 0, z = 0;
    D3() {}
    D3(double a, double b, double c) : x(a), y(b), z(c) {}
    D3 operator+(const D3& o) const { return D3(x + o.x, y + o.y, z + o.z); }
    D3 operator-(const D3& o) const { return D3(x - o.x, y - o.y, z - o.z); }
    D3 operator-() const { return D3(-x, -y, -z); }
    D3 operator*(double d) const { return D3(x * d, y * d, z * d); }
    D3 operator/(double d) const { return D3(x / d, y / d, z / d); }
    double dot(const D3& o) const { return x * o.x + y * o.y + z * o.z; }
    D3 cross(const D3& o) const { return D3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x); }
    double mag() const { return std::sqrt(x * x + y * y + z * z); }
    D3 normalize() const { double m = mag(); return m == 0 ? D3() : D3(x / m, y / m, z / m); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    void basis(D3* u, D3* w) const {  // Vec3::getPerpendicularBasis (Math/src/Vec3.h:53-57)
        D3 a1(1, 0, 0), a2(0, 1, 0);
        *u = (std::abs(dot(a1)) < std::abs(dot(a2))) ? cross(a1).normalize() : cross(a2).normalize();
        *w = cross(*u).normalize();
    }
};

struct HullPrep {
    std::vector<D3> pts;
    D3 interior;
    std::vector<std::vector<int>> faces;
    std::vector<int> nci, dir;
    std::vector<std::pair<int, int>> edges;
    std::vector<std::vector<int>> vfaces, vedges;
    std::vector<D3> gn;
    std::vector<uint8_t> redundant;
    std::vector<int> cmax_id, cmin_id, ref_idx;
    std::vector<double> cmax, cmin, ref_val;
    std::vector<std::pair<int, int>> arcs;

    D3 faceNormal(int f) const {
        const std::vector<int>& s = faces[f];
        D3 p1 = pts[s[0]], p2 = pts[s[1]], p3 = pts[s[nci[f]]];
        return (p2 - p1).cross(p3 - p2).normalize() * (double)dir[f];
    }

    void normalInfo(int f, const D3& normalish) {
        const std::vector<int>& s = faces[f];
        D3 p0 = pts[s[0]], p1 = pts[s[1]];
        int k = 2;
        D3 v1 = (p1 - p0).normalize();
        D3 v2 = (pts[s[k]] - p0).normalize();
        while (std::abs(v1.dot(v2)) > 0.99 && k + 1 < (int)s.size()) v2 = (pts[s[++k]] - p0).normalize();
        nci[f] = k;
        dir[f] = 1;
        if (normalish.dot(faceNormal(f)) < 0) dir[f] = -1;
    }

    void wind(int f, const D3& n) {
        D3 u, w;
        n.basis(&u, &w);
        std::vector<int>& s = faces[f];
        int np = (int)s.size();
        double area = 0;
        for (int i = 0; i < np; i++) {
            D3 a = pts[s[i]], b = pts[s[(i + 1 == np) ? 0 : i + 1]];
            area += (b.dot(w) - a.dot(w)) * (b.dot(u) + a.dot(u)) / 2.0;
        }
        if (area < 0) {
            std::reverse(s.begin(), s.end());
            normalInfo(f, n);
        }
    }

    void extrema(const D3& axis, int* mn_id, double* mn, int* mx_id, double* mx) const {
        *mn = std::numeric_limits<double>::infinity();
        *mx = -std::numeric_limits<double>::infinity();
        *mn_id = *mx_id = -1;
        for (int i = 0; i < (int)pts.size(); i++) {
            double v = pts[i].dot(axis);
            if (v < *mn) { *mn = v; *mn_id = i; }
            if (v > *mx) { *mx = v; *mx_id = i; }
        }
    }

    bool build(const std::vector<D3>& p, const std::vector<std::vector<int>>& f) {
        pts = p;
        int nf = (int)f.size();
        interior = D3();
        for (const D3& q : pts) interior = interior + q;
        interior = interior / (double)pts.size();
        faces = f;
        nci.assign(nf, 2);
        dir.assign(nf, 1);
        vfaces.assign(pts.size(), {});
        vedges.assign(pts.size(), {});
        for (int i = 0; i < nf; i++) {
            if (faces[i].size() < 3) return false;
            for (int j : faces[i]) {
                if (j < 0 || j >= (int)pts.size()) return false;
                vfaces[j].push_back(i);
            }
            normalInfo(i, pts[faces[i][0]] - interior);
            wind(i, faceNormal(i));
        }
        for (int i = 0; i < nf; i++) {
            int n = (int)faces[i].size();
            for (int k = 0; k < n; k++) {
                int a = faces[i][k], b = faces[i][(k + 1) % n];
                bool seen = false;
                for (auto& e : edges) if ((e.first == a && e.second == b) || (e.first == b && e.second == a)) { seen = true; break; }
                if (!seen) edges.push_back({a, b});
            }
        }
        for (int i = 0; i < (int)edges.size(); i++) { vedges[edges[i].first].push_back(i); vedges[edges[i].second].push_back(i); }
        for (int i = 0; i < nf; i++) {
            D3 n = faceNormal(i);
            bool red = false;
            for (const D3& g : gn) if (n.dot(g) < -1 + 0.0000000001) { red = true; break; }
            int mn_id, mx_id;
            double mn, mx;
            extrema(n, &mn_id, &mn, &mx_id, &mx);
            gn.push_back(n);
            redundant.push_back(red);
            cmax_id.push_back(mx_id); cmin_id.push_back(mn_id);
            cmax.push_back(mx); cmin.push_back(mn);
            ref_idx.push_back(faces[i][0]);
            ref_val.push_back(n.dot(pts[faces[i][0]]));
            for (int j = i + 1; j < nf; j++) {
                const std::vector<int>& s1 = faces[i];
                const std::vector<int>& s2 = faces[j];
                for (size_t k = 0; k < s1.size(); k++)
                    for (size_t w = 0; w < s2.size(); w++) {
                        int a1 = s1[k], a2 = s1[(k + 1) % s1.size()], b1 = s2[w], b2 = s2[(w + 1) % s2.size()];
                        if ((a1 == b1 && a2 == b2) || (a1 == b2 && a2 == b1)) { arcs.push_back({i, j}); break; }
                    }
            }
        }
        return true;
    }
};

// Mass properties of a convex polyhedron (volume, centre of mass and inertia
// tensor about the centre of mass, density-weighted) by a fan of tetrahedra
// from the interior point.  The reference integrates the same quantities with
// Mirtich's surface-integral method (RigidBody.cpp:427-640); both are exact
// for polyhedra, so results agree to rounding.
inline void hullMassProperties(const HullPrep& h, double density, D3* com, double tensor[3][3], double* mass) {
    double vol = 0;
    D3 first;
    double c[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    D3 o = h.interior;
    for (const std::vector<int>& s : h.faces) {
        for (size_t t = 1; t + 1 < s.size(); t++) {
            D3 p[4] = {o, h.pts[s[0]], h.pts[s[t]], h.pts[s[t + 1]]};
            double v = (p[1] - p[0]).dot((p[2] - p[0]).cross(p[3] - p[0])) / 6.0;
            D3 sum = p[0] + p[1] + p[2] + p[3];
            vol += v;
            first = first + sum * (v / 4.0);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    double acc = sum[i] * sum[j];
                    for (int k = 0; k < 4; k++) acc += p[k][i] * p[k][j];
                    c[i][j] += v / 20.0 * acc;
                }
        }
    }
    *mass = density * vol;
    *com = first * density / *mass;
    double tr = c[0][0] + c[1][1] + c[2][2];
    double cc[3] = {com->x, com->y, com->z};
    double c2 = com->dot(*com);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            tensor[i][j] = density * ((i == j ? tr : 0.0) - c[i][j]) - *mass * ((i == j ? c2 : 0.0) - cc[i] * cc[j]);
}

}  // namespace cpgpu
