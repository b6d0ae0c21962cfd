/*
 * facade_advance.cpp -- a C++ program written against bbg_bubbles.hpp (the reference's
 * PciSphSolver3 / SphSolver3 API over libbbg): it reads a scene and particles, runs
 * Initialize, Setup, SetColliders and Advance(dt) `count` times, and writes the particles.
 *
 *   facade_advance <in.bin> <out.bin>
 * in.bin (native byte order): int32 n, kind (0 PCISPH, 1 SPH), mode, count; float64 mass,
 * spacing, dt, domain min[3], max[3]; int32 colliders; per collider int32 type, reverse,
 * float64 center[3], size[3]; then n x 3 float64 positions.
 * out.bin: n x 3 float64 positions, n x 3 float64 velocities, int32 substeps of the last
 * Advance.  Exit status: 0, or the bbg status of the failing call.
 */
#include <bbg_bubbles.hpp>

#include <cstdint>
#include <cstdio>
#include <vector>

using namespace bbg_bubbles;

template <class T>
static bool get(FILE *f, T *v, size_t n = 1) {
    return fread(v, sizeof(T), n, f) == n;
}

int main(int argc, char **argv) {
    if (argc != 3) return 64;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 65;
    int32_t n, kind, mode, count, ncol;
    double mass, spacing, dt, lo[3], hi[3];
    if (!get(f, &n) || !get(f, &kind) || !get(f, &mode) || !get(f, &count) || !get(f, &mass) || !get(f, &spacing) ||
        !get(f, &dt) || !get(f, lo, 3) || !get(f, hi, 3) || !get(f, &ncol))
        return 66;
    ColliderSet3 colliders;
    for (int i = 0; i < ncol; i++) {
        int32_t type, reverse;
        double c[3], s[3];
        if (!get(f, &type) || !get(f, &reverse) || !get(f, c, 3) || !get(f, s, 3)) return 66;
        if (type == BBG_SHAPE_BOX) colliders.AddBox(vec3f(c[0], c[1], c[2]), vec3f(s[0], s[1], s[2]), reverse != 0);
        else colliders.AddSphere(vec3f(c[0], c[1], c[2]), s[0]);
    }
    std::vector<double> xyz(3 * (size_t)n);
    if (!get(f, xyz.data(), xyz.size())) return 66;
    fclose(f);
    std::vector<vec3f> pos((size_t)n);
    for (int i = 0; i < n; i++) pos[(size_t)i] = vec3f(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    SphParticleSet3 set(pos);
    set.SetMass(mass);
    Grid3 domain = UtilBuildGridForDomain(Bounds3f{vec3f(lo[0], lo[1], lo[2]), vec3f(hi[0], hi[1], hi[2])}, spacing, 2.0);
    int substeps = 0;
    try {
        SphSolverData3 data = DefaultSphSolverData3(true);
        data.gravity = vec3f(0.0, -9.81, 0.0);
        if (kind == 0) {
            PciSphSolver3 solver;
            solver.pcisphMode = mode;
            solver.maxIterations = mode == BBG_PCISPH_AS_SHIPPED ? 5 : 20;
            solver.Initialize(data);
            solver.Setup(1000.0, spacing, 2.0, domain, &set);
            solver.SetColliders(colliders);
            for (int k = 0; k < count; k++) solver.Advance(dt);
            substeps = solver.GetLastStats().substeps;
            printf("PciSphSolver3: %d particles, last Advance %d substeps, %.3f ms\n", solver.GetParticleCount(),
                   substeps, solver.GetAdvanceTime());
        } else {
            SphSolver3 solver;
            solver.Initialize(data);
            solver.Setup(1000.0, spacing, 2.0, domain, &set);
            solver.SetColliders(colliders);
            for (int k = 0; k < count; k++) solver.Advance(dt);
            substeps = solver.GetLastStats().substeps;
            printf("SphSolver3: %d particles, last Advance %d substeps\n", solver.GetParticleCount(), substeps);
        }
    } catch (const Error &e) {
        fprintf(stderr, "%s\n", e.what());
        return e.status;
    }
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 67;
    for (int i = 0; i < n; i++) {
        const vec3f p = set.GetParticlePosition(i);
        const double v[3] = {p.x, p.y, p.z};
        fwrite(v, sizeof(double), 3, o);
    }
    for (int i = 0; i < n; i++) {
        const vec3f p = set.GetParticleVelocity(i);
        const double v[3] = {p.x, p.y, p.z};
        fwrite(v, sizeof(double), 3, o);
    }
    const int32_t s = substeps;
    fwrite(&s, sizeof(s), 1, o);
    fclose(o);
    return 0;
}
