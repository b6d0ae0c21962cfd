/*
 * bbg_bubbles.hpp -- the reference's C++ solver API (class and method names, argument
 * meaning, call order) over the bbg C ABI, header-only, C++17.
 *
 * A program written against Bubbles' PciSphSolver3 / SphSolver3 (src/core/pcisph_solver.h:
 * 56-83, src/core/sph_solver.h:76-96) keeps its structure:
 *
 *     bbg_bubbles::PciSphSolver3 solver;
 *     solver.Initialize(bbg_bubbles::DefaultSphSolverData3());       // sph_solver3.cpp:124-151
 *     bbg_bubbles::SphParticleSet3 set(positions);                   // ParticleSetBuilder3 output
 *     bbg_bubbles::Grid3 domain = bbg_bubbles::UtilBuildGridForDomain(bounds, spacing, 2.0);
 *     solver.Setup(1000.0, spacing, 2.0, domain, &set);              // pcisph_solver3.cpp:103-146
 *     solver.SetColliders(colliders);                                // MakeBox / MakeSphere shapes
 *     solver.Advance(dt);                                            // pcisph_solver3.cpp:67-89
 *
 * The particle set keeps the reference's FP64 AoS positions and velocities on the host;
 * Advance runs the CFL substeps on the device and copies the state back into the set.
 * Differences from the reference, each deliberate: errors throw bbg_bubbles::Error
 * (the reference asserts or exits); the corrector defaults to the reference's as-shipped
 * behaviour and `pcisphMode = BBG_PCISPH_TOLERANCE` makes maxIterations and
 * maxErrorDensity take effect (the reference hard-codes 5 and 0.01 at its call site,
 * pcisph_solver3.cpp:62-63); colliders are analytic boxes and spheres with
 * translation-only transforms; GetAdvanceTime is the wall time of the last Advance in
 * milliseconds.
 */
#ifndef BBG_BUBBLES_HPP
#define BBG_BUBBLES_HPP

#include <chrono>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bbg.h"

namespace bbg_bubbles {

using Float = double;

struct vec3f {
    Float x = 0, y = 0, z = 0;
    vec3f() = default;
    vec3f(Float a, Float b, Float c) : x(a), y(b), z(c) {}
    Float operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};

struct Bounds3f {
    vec3f pMin, pMax;
};

class Error : public std::runtime_error {
public:
    Error(bbg_status status, const std::string &what) : std::runtime_error(what), status(status) {}
    bbg_status status;
};

inline void Check(bbg_status st, const char *call) {
    if (st != BBG_OK) throw Error(st, std::string(call) + ": " + bbg_last_error());
}

/* SphSolverData3's scalar settings (sph_solver.h:31-50) with DefaultSphSolverData3's values. */
struct SphSolverData3 {
    Float eosExponent = 7.0;
    Float negativePressureScale = 0.0;
    Float viscosity = 0.04;
    Float pseudoViscosity = 10.0;
    Float soundSpeed = 100.0;
    Float dragCoefficient = 0.0001;
    vec3f gravity{0.0, -9.8, 0.0};   /* the constant interaction AddConstantInteraction adds */
};

inline SphSolverData3 DefaultSphSolverData3(bool with_gravity = true) {
    SphSolverData3 d;
    if (!with_gravity) d.gravity = vec3f(0.0, 0.0, 0.0);
    return d;
}

/* SphParticleSet3 over a ParticleSet3 (particle.h:154-401, 508-609): positions and
 * velocities (FP64, as the reference stores them) and the mass; Setup fills the SPH
 * settings.  A mass <= 0 lets Setup compute it as the reference's ComputeMass does. */
class SphParticleSet3 {
public:
    explicit SphParticleSet3(std::vector<vec3f> positions, std::vector<vec3f> velocities = {})
        : pos_(std::move(positions)), vel_(std::move(velocities)) {
        if (vel_.empty()) vel_.resize(pos_.size());
        if (vel_.size() != pos_.size()) throw Error(BBG_ERR_INVALID_ARGUMENT, "SphParticleSet3: size mismatch");
    }
    int GetParticleCount() const { return (int)pos_.size(); }
    vec3f GetParticlePosition(int i) const { return pos_.at((size_t)i); }
    vec3f GetParticleVelocity(int i) const { return vel_.at((size_t)i); }
    void SetParticlePosition(int i, vec3f p) { pos_.at((size_t)i) = p; }
    void SetParticleVelocity(int i, vec3f v) { vel_.at((size_t)i) = v; }
    void SetMass(Float m) { mass_ = m; }
    Float GetMass() const { return mass_; }
    Float GetTargetDensity() const { return density_; }
    Float GetTargetSpacing() const { return spacing_; }
    Float GetKernelRadius() const { return spacing_ * relative_; }

private:
    friend class SolverBase;
    std::vector<vec3f> pos_, vel_;
    Float mass_ = 0, density_ = 1000.0, spacing_ = 0, relative_ = 2.0;
};

/* The domain grid of UtilBuildGridForDomain (util.cpp:269-287): the bounds it is built
 * over and the cell length spacing x spacingScale. */
class Grid3 {
public:
    Grid3(Bounds3f bounds, Float spacing, Float spacingScale) : bounds_(bounds), spacing_(spacing), scale_(spacingScale) {
        const double lo[3] = {bounds.pMin.x, bounds.pMin.y, bounds.pMin.z};
        const double hi[3] = {bounds.pMax.x, bounds.pMax.y, bounds.pMax.z};
        double geo[12];
        Check(bbg_build_grid(lo, hi, spacing, spacingScale, dims_, geo), "bbg_build_grid");
    }
    /* GetIndexCount: cells per axis */
    const int *GetIndexCount() const { return dims_; }
    int GetCellCount() const { return dims_[0] * dims_[1] * dims_[2]; }
    const Bounds3f &GetDomainBounds() const { return bounds_; }
    Float GetSpacingScale() const { return scale_; }
    Float GetSpacing() const { return spacing_; }

private:
    Bounds3f bounds_;
    Float spacing_, scale_;
    int dims_[3] = {0, 0, 0};
};

inline Grid3 UtilBuildGridForDomain(Bounds3f bounds, Float spacing, Float spacingScale = 2.0) {
    return Grid3(bounds, spacing, spacingScale);
}

/* ColliderSet3 (collider.cpp:238-264) of MakeBox(Translate(c), size, reverse) and
 * MakeSphere(Translate(c), radius) shapes. */
class ColliderSet3 {
public:
    void AddBox(vec3f center, vec3f size, bool reverseOrientation, Float friction = 0.0) {
        shapes_.push_back(shape(BBG_SHAPE_BOX, reverseOrientation, center, size, friction));
    }
    void AddSphere(vec3f center, Float radius, Float friction = 0.0) {
        shapes_.push_back(shape(BBG_SHAPE_SPHERE, false, center, vec3f(radius, 0, 0), friction));
    }
    const std::vector<bbg_shape> &Shapes() const { return shapes_; }

private:
    static bbg_shape shape(int type, bool reverse, vec3f c, vec3f s, Float friction) {
        bbg_shape sh{};
        sh.type = type;
        sh.reverse = reverse ? 1 : 0;
        for (int k = 0; k < 3; k++) {
            sh.center[k] = c[k];
            sh.size[k] = s[k];
        }
        sh.friction = friction;
        return sh;
    }
    std::vector<bbg_shape> shapes_;
};

/* What PciSphSolver3 and SphSolver3 share: the device solver, its description and the
 * particle set it advances. */
class SolverBase {
public:
    SolverBase(const SolverBase &) = delete;
    SolverBase &operator=(const SolverBase &) = delete;
    virtual ~SolverBase() {
        if (h_) bbg_destroy(h_);
    }
    void Initialize(const SphSolverData3 &data) {
        data_ = data;
        initialized_ = true;
    }
    void Setup(Float targetDensity, Float targetSpacing, Float relativeRadius, const Grid3 &domain,
               SphParticleSet3 *pSet) {
        if (!initialized_ || !pSet) throw Error(BBG_ERR_STATE, "Setup: Initialize first, with a particle set");
        bbg_solver_desc d;
        Check(bbg_solver_desc_default(&d, kind_), "bbg_solver_desc_default");
        d.eos_exponent = data_.eosExponent;
        d.negative_pressure_scale = data_.negativePressureScale;
        d.viscosity = data_.viscosity < 0 ? 0 : data_.viscosity;
        d.pseudo_viscosity = data_.pseudoViscosity;
        d.sound_speed = data_.soundSpeed;
        d.drag_coefficient = data_.dragCoefficient;
        for (int k = 0; k < 3; k++) {
            d.gravity[k] = data_.gravity[k];
            d.domain_min[k] = domain.GetDomainBounds().pMin[k];
            d.domain_max[k] = domain.GetDomainBounds().pMax[k];
        }
        d.target_density = targetDensity;
        d.target_spacing = targetSpacing;
        d.relative_kernel_radius = relativeRadius;
        d.grid_spacing_scale = domain.GetSpacingScale();
        d.mass = pSet->mass_;
        configure(&d);
        if (h_) bbg_destroy(h_);
        h_ = nullptr;
        set_ = pSet;
        const int n = pSet->GetParticleCount();
        Check(bbg_create(&d, n, &h_), "bbg_create");
        if (!colliders_.empty())
            Check(bbg_set_colliders(h_, colliders_.data(), (int)colliders_.size()), "bbg_set_colliders");
        upload();
        Check(bbg_setup(h_), "bbg_setup");
        double sc[8];
        Check(bbg_get_scalars(h_, sc), "bbg_get_scalars");
        pSet->mass_ = sc[0];
        pSet->density_ = targetDensity;
        pSet->spacing_ = targetSpacing;
        pSet->relative_ = relativeRadius;
    }
    void SetColliders(const ColliderSet3 &colliders) {
        colliders_ = colliders.Shapes();
        if (h_) Check(bbg_set_colliders(h_, colliders_.data(), (int)colliders_.size()), "bbg_set_colliders");
    }
    /* Substeps of the CFL count until the interval is covered, on the device; the particle
     * set holds the new state afterwards. */
    void Advance(Float timeIntervalInSeconds) {
        require();
        const auto t0 = std::chrono::steady_clock::now();
        bbg_step_stats st;
        Check(bbg_advance(h_, timeIntervalInSeconds, &st), "bbg_advance");
        download();
        last_stats_ = st;
        advance_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    /* Positions and velocities changed in the set since Setup or the last Advance go to the
     * device (the grid is rebuilt at the next substep). */
    void PushParticleSet() {
        require();
        upload();
    }
    Float GetAdvanceTime() const { return advance_ms_; }
    int GetParticleCount() const { return set_ ? set_->GetParticleCount() : 0; }
    SphParticleSet3 *GetSphParticleSet() { return set_; }
    const bbg_step_stats &GetLastStats() const { return last_stats_; }
    bbg_solver Handle() const { return h_; }

protected:
    explicit SolverBase(int kind) : kind_(kind) {}
    virtual void configure(bbg_solver_desc *) {}
    void require() const {
        if (!h_ || !set_) throw Error(BBG_ERR_STATE, "call Setup first");
    }
    void upload() {
        const size_t n = set_->pos_.size();
        std::vector<float> p(3 * n), v(3 * n);
        for (size_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                p[3 * i + k] = (float)set_->pos_[i][k];
                v[3 * i + k] = (float)set_->vel_[i][k];
            }
        Check(bbg_upload_particles(h_, p.data(), v.data(), (int)n), "bbg_upload_particles");
    }
    void download() {
        const size_t n = set_->pos_.size();
        std::vector<float> p(3 * n), v(3 * n);
        Check(bbg_download(h_, p.data(), v.data()), "bbg_download");
        for (size_t i = 0; i < n; i++) {
            set_->pos_[i] = vec3f(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
            set_->vel_[i] = vec3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        }
    }
    int kind_;
    bool initialized_ = false;
    SphSolverData3 data_;
    std::vector<bbg_shape> colliders_;
    SphParticleSet3 *set_ = nullptr;
    bbg_solver h_ = nullptr;
    bbg_step_stats last_stats_{};
    double advance_ms_ = 0;
};

/* PciSphSolver3 (pcisph_solver.h:56-83). */
class PciSphSolver3 : public SolverBase {
public:
    Float maxErrorDensity = 0.01;
    unsigned int maxIterations = 5;
    int pcisphMode = BBG_PCISPH_AS_SHIPPED;

    PciSphSolver3() : SolverBase(BBG_SOLVER_PCISPH) {}
    void SetViscosityCoefficient(Float viscosityCoefficient) {
        data_.viscosity = viscosityCoefficient < 0 ? 0 : viscosityCoefficient;
    }
    /* ComputeDelta / ComputeBeta / ComputeDeltaDenom (pcisph_solver3.cpp:148-189). */
    Float ComputeDelta(Float timeIntervalInSeconds) {
        require();
        double d = 0;
        Check(bbg_compute_delta(h_, timeIntervalInSeconds, &d), "bbg_compute_delta");
        return d;
    }
    Float ComputeDeltaDenom() {
        require();
        double sc[8];
        Check(bbg_get_scalars(h_, sc), "bbg_get_scalars");
        return sc[2];
    }
    Float ComputeBeta(Float timeIntervalInSeconds) {
        require();
        double sc[8];
        Check(bbg_get_scalars(h_, sc), "bbg_get_scalars");
        return 2.0 * sc[3] * timeIntervalInSeconds * timeIntervalInSeconds;
    }

protected:
    void configure(bbg_solver_desc *d) override {
        d->pcisph_mode = pcisphMode;
        d->max_iterations = (int)maxIterations;   /* as shipped: one pass, whatever the cap */
        d->max_density_error_ratio = maxErrorDensity;
        d->time_step_limit_scale = 5.0;   /* kDefaultTimeStepLimitScale */
    }
};

/* SphSolver3 (sph_solver.h:76-96). */
class SphSolver3 : public SolverBase {
public:
    SphSolver3() : SolverBase(BBG_SOLVER_SPH) {}
    void SetViscosityCoefficient(Float viscosityCoefficient) {
        data_.viscosity = viscosityCoefficient < 0 ? 0 : viscosityCoefficient;
    }
    void SetPseudoViscosityCoefficient(Float pseudoViscosityCoefficient) {
        data_.pseudoViscosity = pseudoViscosityCoefficient < 0 ? 0 : pseudoViscosityCoefficient;
    }
    Float GetKernelRadius() const { return set_ ? set_->GetKernelRadius() : 0; }

protected:
    void configure(bbg_solver_desc *d) override { d->time_step_limit_scale = 1.0; }
};

}  // namespace bbg_bubbles

#endif
