// Orbital elements and small 3-vectors for the host side.
#pragma once
#include <cmath>

namespace glisser {

struct Vec3 {
    double x, y, z;
    Vec3 operator+(const Vec3& b) const { return { x + b.x, y + b.y, z + b.z }; }
    Vec3 operator-(const Vec3& b) const { return { x - b.x, y - b.y, z - b.z }; }
    Vec3 operator*(double s) const { return { x * s, y * s, z * s }; }
    Vec3 operator/(double s) const { return { x / s, y / s, z / s }; }
    Vec3& operator+=(const Vec3& b) { x += b.x; y += b.y; z += b.z; return *this; }
    Vec3& operator-=(const Vec3& b) { x -= b.x; y -= b.y; z -= b.z; return *this; }
    double lensq() const { return x * x + y * y + z * z; }
};

struct Elements {
    int esign;                      // -1 ellipse, 0 parabola, 1 hyperbola
    double a, e, i, capom, om, f;   // f: true anomaly
};

double ecc_anomaly(double e, double M);
void from_elements(double mu, double a, double e, double i, double capom, double om, double f, Vec3& r, Vec3& v);
void from_elements_M(double mu, double a, double e, double i, double capom, double om, double M, Vec3& r, Vec3& v);
Elements to_elements(double mu, const Vec3& r, const Vec3& v);
double mean_anomaly(double e, double f);

}  // namespace glisser
