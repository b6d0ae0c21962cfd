// host_math.cpp -- host-side setup math of the solver, in the reference's FP32
// arithmetic (Float = float, with its double-precision literals).  Compiled with
// -ffp-contract=off so x86-64 and aarch64 hosts produce identical grids and masses.
#include "host_math.h"

#include <cfloat>
#include <cmath>
#include <vector>

namespace bbg {
namespace {

struct f3 { float x, y, z; };
inline f3 mk(float x, float y, float z) { return f3{x, y, z}; }
inline float axis(const f3 &a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline float lmin(float a, float b) { return a < b ? a : b; }
inline float lmax(float a, float b) { return a < b ? b : a; }
inline float labs(float v) { return v > 0 ? v : -v; }
inline bool is_zero(float a) { return (double)labs(a) < 1e-8; }
inline float length(f3 a) { return (float)std::sqrt((double)(a.x * a.x + a.y * a.y + a.z * a.z)); }

constexpr double kPi = 3.14159265358979323846;

// SphStdKernel3::W, src/core/kernel.cpp:123-132
float std_w(float h, float distance) {
    float h2 = h * h, h3 = h2 * h;
    float d2 = distance * distance;
    float of = d2 - h2;
    if (is_zero(of) || of > 0) return 0;
    float x = 1.0 - d2 / h2;
    return 315.0 / (64.0 * kPi * h3) * x * x * x;
}

// SphSpikyKernel3::dW, src/core/kernel.cpp:191-199
float spiky_dw(float h, float distance) {
    float h2 = h * h, h4 = h2 * h2;
    float of = distance - h;
    if (is_zero(of) || of > 0) return 0;
    float x = 1.0 - distance / h;
    return -45.0 / (kPi * h4) * x * x;
}

// Lattice points covering [-1.5 r, 1.5 r]^3.  kind 0: BccLatticePointGenerator
// (src/generator/bcclattice.cpp:5-77); kind 1: simple cubic with the same loop bounds.
std::vector<f3> lattice(int kind, float spacing, float kernelRadius, size_t maxn) {
    float a = -1.5 * kernelRadius, b = 1.5 * kernelRadius;
    f3 mn = mk(lmin(a, b), lmin(a, b), lmin(a, b));
    f3 mx = mk(lmax(a, b), lmax(a, b), lmax(a, b));
    float halfSpacing = spacing / 2;
    float width = labs(mx.x - mn.x), height = labs(mx.y - mn.y), depth = labs(mx.z - mn.z);
    std::vector<f3> pts;
    bool hasOff = false, stop = false;
    float zstep = kind == 0 ? halfSpacing : spacing;
    for (int k = 0; k * zstep <= depth && !stop; k++) {
        float z = k * zstep + mn.z;
        float offset = (kind == 0 && hasOff) ? halfSpacing : 0;
        for (int j = 0; j * spacing + offset <= height && !stop; j++) {
            float y = j * spacing + offset + mn.y;
            for (int i = 0; i * spacing + offset <= width && !stop; i++) {
                float x = i * spacing + offset + mn.x;
                if (pts.size() < maxn) pts.push_back(mk(x, y, z));
                else { stop = true; break; }
            }
        }
        hasOff = !hasOff;
    }
    return pts;
}

}  // namespace

// UtilBuildGridForDomain (src/core/util.cpp:269-287) + Grid::Build (src/core/grid.h:627-666)
void build_grid(const double dmin[3], const double dmax[3], double spacing_d, double scale_d,
                int dims[3], float minp[3], float len[3], float bmin[3], float bmax[3]) {
    float spacing = (float)spacing_d, spacingScale = (float)scale_d;
    f3 a = mk((float)dmin[0], (float)dmin[1], (float)dmin[2]);
    f3 b = mk((float)dmax[0], (float)dmax[1], (float)dmax[2]);
    f3 dlo = mk(lmin(a.x, b.x), lmin(a.y, b.y), lmin(a.z, b.z));
    f3 dhi = mk(lmax(a.x, b.x), lmax(a.y, b.y), lmax(a.z, b.z));
    float length = spacing * spacingScale;
    float hlen = 0.5 * length;
    float invLen = 1.0f / length;
    int m[3];
    for (int k = 0; k < 3; k++) {
        m[k] = (int)std::ceil(labs(axis(dhi, k) - axis(dlo, k)) * invLen);
        m[k] += (m[k] % 2) * length;   // truncates back to m[k] for length < 1, as in the reference
    }
    float half[3] = {m[0] * hlen, m[1] * hlen, m[2] * hlen};
    float center[3];
    for (int k = 0; k < 3; k++) center[k] = (axis(dlo, k) + axis(dhi, k)) * (float)0.5;
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        float p0 = center[k] - half[k], p1 = center[k] + half[k];
        float dl = lmax(p0, p1), du = lmin(p0, p1);
        float l = FLT_MAX, h = -FLT_MAX;
        if (dl < l) l = dl;
        if (dl > h) h = dl;
        if (du > h) h = du;
        if (du < l) l = du;
        lo[k] = l;
        hi[k] = h;
    }
    for (int k = 0; k < 3; k++) {
        float s = hi[k] - lo[k];
        float cl = s / (float)m[k];
        len[k] = cl;
        dims[k] = (int)std::ceil(s / cl);
        float maxp = lo[k] + (float)dims[k] * cl;
        minp[k] = lo[k];
        bmin[k] = lmin(lo[k], maxp);
        bmax[k] = lmax(lo[k], maxp);
    }
}

// SphParticleSet3::ComputeMass (src/core/particle.h:557-582)
float compute_mass(int lattice_kind, float targetDensity, float targetSpacing, float kernelRadius) {
    std::vector<f3> pts = lattice(lattice_kind, targetSpacing, kernelRadius, 1024);
    float nDen = 0;
    for (size_t i = 0; i < pts.size(); i++) {
        float sum = 0;
        for (size_t j = 0; j < pts.size(); j++) {
            f3 d = mk(pts[i].x - pts[j].x, pts[i].y - pts[j].y, pts[i].z - pts[j].z);
            sum += std_w(kernelRadius, length(d));
        }
        nDen = lmax(nDen, sum);
    }
    return targetDensity / nDen;
}

// PciSphSolver3::ComputeDeltaDenom (src/solvers/pcisph_solver3.cpp:148-180)
float compute_delta_denom(float spacing, float kernelRadius) {
    std::vector<f3> pts = lattice(0, spacing, kernelRadius, (size_t)-1);
    float kernelRadius2 = kernelRadius * kernelRadius;
    float denom2 = 0;
    f3 denom1 = mk(0, 0, 0);
    for (const f3 &p : pts) {
        float d2 = p.x * p.x + p.y * p.y + p.z * p.z;
        if (d2 < kernelRadius2) {
            float distance = (float)std::sqrt((double)d2);
            f3 dir = mk(0, 0, 0);
            if (distance > 0) {
                float inv = (float)1 / distance;
                dir = mk(p.x * inv, p.y * inv, p.z * inv);
            }
            float s = -spiky_dw(kernelRadius, distance);
            f3 g = mk(dir.x * s, dir.y * s, dir.z * s);
            denom1 = mk(denom1.x + g.x, denom1.y + g.y, denom1.z + g.z);
            denom2 += g.x * g.x + g.y * g.y + g.z * g.z;
        }
    }
    float denom = 0;
    denom += -(denom1.x * denom1.x + denom1.y * denom1.y + denom1.z * denom1.z) - denom2;
    return denom;
}

// PciSphSolver3::ComputeDelta / ComputeBeta (pcisph_solver3.cpp:182-189)
float compute_delta(float massOverTargetDensitySquared, float deltaDenom, float dt) {
    float timeStepSquare = dt * dt;
    float beta = 2.0 * massOverTargetDensitySquared * timeStepSquare;
    return labs(deltaDenom) > 0 ? -1 / (beta * deltaDenom) : 0;
}

// SphParticleSet3::ComputeNumberOfTimeSteps (particle.h:584-608), given max |F|
unsigned number_of_time_steps(float timeStep, float speedOfSound, float timeStepScale,
                              float kernelRadius, float mass, float maxForce) {
    float refDist = kernelRadius;
    float timeStepLimit = 0.40 * refDist / speedOfSound;
    if (!is_zero(maxForce)) {
        float byForce = 0.25 * std::sqrt((double)(refDist * mass / maxForce));
        timeStepLimit = lmin(byForce, timeStepLimit);
    }
    float targetTimeStep = timeStepScale * timeStepLimit;
    return (unsigned)std::ceil(timeStep / targetTimeStep);
}

// Float threshold T for a double threshold t: for every float x, x < t <=> x < T.
float float_above(double t) {
    float f = (float)t;
    if ((double)f < t) f = std::nextafter(f, FLT_MAX);
    return f;
}

}  // namespace bbg
