// CPU oracle for the WCSPH step of NCCA/libfluid.
//
// TEST INFRASTRUCTURE ONLY.  This file is a CPU restatement of the reference's
// per-substep algorithm (libfluid/cudasrc/fluidsystem.cu:273-399 and the
// kernels it launches).  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / --impl reference legs of bench.py may load it, and only as
// the checker or the timed CPU baseline.  The product library never links,
// loads or calls it.
//
// Two precisions are built from one template:
//   * float  - mirrors the reference's FP32 arithmetic, including its quirks:
//              double-precision sub-expressions (fluidkernel.cu:65,
//              fluidphysics.cu:279), the cohesion precedence bug
//              (fluidkernel.cu:37), the re-added pressure term in the
//              "viscosity" sum (fluidphysics.cu:287), rho_i + rho_i in the
//              tension denominator (fluidphysics.cu:293), the swapped
//              adhesion/viscosity buffers (fluidsystem.cu:352-364 vs
//              fluidphysics.cu:215-219) and the float-accumulated substep
//              loop (fluidsystem.cu:301).
//   * double - the same algorithm in FP64, used to state the error of each
//              FP32 result.
//
// Contraction pattern.  nvcc fuses multiply-adds in the reference build; the
// oracle writes the fused operations out with std::fma at these points
// (compiled with -ffp-contract=off so nothing else is fused):
//   dot(a,b)           = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))
//   h2 - r*r           = fma(-r, r, h2)
//   running sums s+=a*b = fma(a, b, s)
//   acc_next           = fma(force, m, g)
//   pos += v*dt+...    = pos + fma(v, dt, (0.5*a)*dtdt)
//   vel += 0.5(a+a')dt = fma(0.5*(a+a'), dt, vel)
//   pos -= s*n         = fma(-s, n, pos)
// Everything else is evaluated operation by operation in source order.
//
// Deviations from the reference (stated, not hidden):
//   * XSPH (fluidphysics.cu:355-409) updates velocities in place while other
//     threads read them: a data race.  The oracle uses Jacobi semantics: all
//     reads see the post-integration, pre-XSPH velocities.
//   * normalize() (CUDA Samples helper_math, not in the reference tree) is
//     v * rsqrtf(dot(v,v)); the oracle uses v * (1/sqrtf(dot(v,v))).
//   * Particles outside the grid (NULL_HASH, fluiddefines.h:12) are skipped by
//     the neighbour passes and keep stale density/forces in the reference
//     (quirk: whatever the array held at that sorted index).  The oracle gives
//     them zero density, pressure, sound speed, normal and force, which is
//     what the reference arrays hold right after init (fluidsystem.cu:238-251).
//
// Parity pins: see tests/test_oracle.py (known answers restated from the
// reference sources) and tests/golden/ (vectors from the reference's own
// device code, when available).

#include <cstdint>
#include <cstring>
#include <cmath>
#include <cfloat>
#include <climits>
#include <vector>
#include <algorithm>
#include <string>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint32_t NULL_HASH = 0xFFFFFFFFu;      // fluiddefines.h:12 (UINT_MAX)
constexpr float PI_F = 3.141592654f;             // fluiddefines.h:16 (CUDART_PI_F)

template <class T> struct V3 { T x, y, z; };
template <class T> inline V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> inline V3<T> operator-(V3<T> a) { return mk(-a.x, -a.y, -a.z); }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return mk(s * a.x, s * a.y, s * a.z); }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return mk(a.x / s, a.y / s, a.z / s); }
template <class T> inline T fma_(T a, T b, T c) { return std::fma(a, b, c); }
// helper_math's dot (a.x*b.x + a.y*b.y + a.z*b.z) with the multiply-add
// fusion of the reference's nvcc build: the x product into the first add,
// the z product into the second (pinned by the reference-built goldens).
template <class T> inline T dot(V3<T> a, V3<T> b) { return fma_(a.z, b.z, fma_(a.x, b.x, a.y * b.y)); }
template <class T> inline T sqrt_(T x) { return std::sqrt(x); }
// magnitude in double (test scales only)
template <class T> inline double vnorm(V3<T> a) {
    return std::sqrt(double(a.x) * double(a.x) + double(a.y) * double(a.y) + double(a.z) * double(a.z));
}
template <class T> inline T pow_(T x, T y) { return std::pow(x, y); }
template <class T> inline V3<T> fmaV(V3<T> a, T s, V3<T> c) { return mk(fma_(a.x, s, c.x), fma_(a.y, s, c.y), fma_(a.z, s, c.z)); }
template <class T> inline V3<T> fmaV(T s, V3<T> a, V3<T> c) { return mk(fma_(s, a.x, c.x), fma_(s, a.y, c.y), fma_(s, a.z, c.z)); }

// float -> int conversion with the device semantics of cvt.rzi.s32.f32
// (round toward zero, saturate, NaN -> 0): grid_from_point (fluidutil.cu:15-18)
// converts floor(p*res) to int on the GPU.
template <class T> inline int32_t f2i_dev(T v) {
    if (v != v) return 0;
    if (v >= T(2147483647.0)) return INT32_MAX;
    if (v <= T(-2147483648.0)) return INT32_MIN;
    return (int32_t)v;
}

// Derived parameter block.  Mirrors FluidParamData (fluidparams.cuh:16-69)
// plus the generalised domain (box extents and grid dims per axis).  In the
// reference the domain is the unit cube with h = 1/res (fluidparams.cu:62).
template <class T> struct Params {
    uint32_t res = 0, gx = 1, gy = 1, gz = 1, numCells = 1;
    T inv_cell = T(1);                 // cell scale: grid = floor(p * inv_cell)
    V3<T> box_c{T(0.5), T(0.5), T(0.5)}, box_b{T(0.5), T(0.5), T(0.5)};
    // boundary shape: 0 the box (the reference's boundarySDF), 1 the sphere of
    // radius min(box_b) about box_c that boundarySDF computes but does not
    // return (fluidutil.cu:97-99)
    int boundary = 0;
    uint32_t numParticles = 0;
    T restDensity{}, invRestDensity{}, gasConstant{}, gamma{}, invGamma{};
    T mass{}, mass2{}, invMass{}, particleSize{}, invParticleSize{};
    T dt{}, dtdt{};
    T h{}, halfh{}, h2{}, h3{}, h4{}, h5{}, h6{}, h8{}, h9{}, invh{}, invh2{}, invh3{}, invh6{}, invh9{};
    T xsph{}, surfaceTension{}, viscosity{}, adhesion{};
    T velLimit{}, accLimit{}, velLimit2{}, accLimit2{};
    T vdamp{};
    V3<T> gravity{T(0), T(-9.8), T(0)};
    T poly6{}, gradPoly6{}, lapPoly6{}, spiky{}, gradSpiky{}, lapVisc{}, cohesion{};
    T eps{};
};

// Smoothing-length-derived constants: FluidParams::setRes (fluidparams.cu:51-89).
template <class T> void derive_h(Params<T>& p, T h) {
    p.h = h;
    p.halfh = T(0.5) * h;
    p.h2 = h * h;
    p.h3 = h * h * h;
    p.h4 = h * h * h * h;
    p.h5 = p.h3 * p.h2;
    p.h6 = p.h3 * p.h3;
    p.h8 = p.h5 * p.h3;
    p.h9 = p.h6 * p.h3;
    p.invh = T(1) / h;
    p.invh2 = T(1) / p.h2;
    p.invh3 = T(1) / p.h3;
    p.invh6 = T(1) / p.h6;
    p.invh9 = T(1) / (p.h6 * p.h3);
    const T pi = T(PI_F);
    p.poly6 = T(315) / (T(64) * pi * pow_(p.h, T(9)));
    p.gradPoly6 = T(-945) / (T(32) * pi * pow_(p.h, T(9)));
    p.lapPoly6 = T(-945) / (T(32) * pi * pow_(p.h, T(9)));
    p.spiky = T(15) / (pi * pow_(p.h, T(6)));
    p.gradSpiky = T(-45) / (pi * pow_(p.h, T(6)));
    p.lapVisc = T(45) / (pi * pow_(p.h, T(6)));
    p.cohesion = T(32) / (pi * pow_(p.h, T(9)));
}

template <class T> void set_res(Params<T>& p, uint32_t res) {
    // fluidparams.cu:53-54: res 0 or unchanged res is ignored.
    if (res == 0 || res == p.res) return;
    p.res = res;
    p.gx = p.gy = p.gz = res;
    p.numCells = res * res * res;
    p.inv_cell = T(float(res));           // grid_from_point multiplies by m_res (fluidutil.cu:17)
    p.box_c = mk(T(0.5f), T(0.5f), T(0.5f));
    p.box_b = p.box_c;
    derive_h(p, T(1.0f / float(res)));    // fluidparams.cu:62 (computed in float)
}
template <class T> void set_rest_density(Params<T>& p, T v) { p.restDensity = v; p.invRestDensity = (v == T(0)) ? T(1) : T(1) / v; }
template <class T> void set_gamma(Params<T>& p, T v) { p.gamma = v; p.invGamma = (v == T(0)) ? T(1) : T(1) / v; }
template <class T> void set_mass(Params<T>& p, T v) { p.mass = v; p.mass2 = v * v; p.invMass = T(1) / v; }
template <class T> void set_psize(Params<T>& p, T v) { p.particleSize = v; p.invParticleSize = T(1) / v; }
template <class T> void set_limits(Params<T>& p, T v, T a) { p.velLimit = v; p.accLimit = a; p.velLimit2 = v * v; p.accLimit2 = a * a; }
template <class T> void set_dt(Params<T>& p, T v) { p.dt = v; p.dtdt = v * v; }

// FluidParams constructor defaults (fluidparams.cuh:81-97, fluidparams.cu:11-49).
template <class T> void ctor_defaults(Params<T>& p) {
    set_res(p, 1u);
    p.numParticles = 1;
    set_rest_density(p, T(1.0f));   // DEFAULT_REST_DENSITY
    p.gasConstant = T(1.0f);        // DEFAULT_GAS_CONSTANT
    set_gamma(p, T(1.0f));
    set_mass(p, T(1.0f));
    set_limits(p, T(5.0f), T(150.0f));
    p.surfaceTension = T(1.0f);     // DEFAULT_SURFACE_TENSION_FORCE
    p.viscosity = T(0.1f);          // DEFAULT_VISCOSITY_FORCE
    p.adhesion = T(1.0f);           // DEFAULT_ADHESION_FORCE
    p.xsph = T(0.5f);
    p.vdamp = T(1.0f);
    set_psize(p, T(1.0f));
    set_dt(p, T(0.01f));            // DEFAULT_TIMESTEP
    p.gravity = mk(T(0.0f), T(-9.8f), T(0.0f));
    p.eps = T(FLT_MIN);             // std::numeric_limits<float>::min() (fluidparams.cu:48)
}

// FluidSystem::init parameter resets (fluidsystem.cu:202-235).
template <class T> void init_defaults(Params<T>& p, uint32_t n, uint32_t res) {
    set_res(p, res);
    p.numParticles = n;
    p.gasConstant = T(100.0f);
    p.vdamp = T(0.0f);
    set_gamma(p, T(7.0f));
    set_limits(p, T(5.0f), T(150.0f));
    set_dt(p, T(1.0f));
    p.xsph = T(0.5f);
    set_psize(p, T(1.0f));
    set_rest_density(p, T(1000.0f));
    set_mass(p, T(1.0f));
}

// Generalised rectangular domain [0,lx]x[0,ly]x[0,lz] with cell size h.  The
// reference's unit cube is the special case lx=ly=lz=1, h=1/res.
template <class T> void set_domain(Params<T>& p, float lx, float ly, float lz, float h) {
    const float inv = 1.0f / h;
    // cells per axis: ceil(l/h), tolerant to the float rounding of h
    auto cells = [&](float l) -> uint32_t {
        double c = std::ceil(double(l) / double(h) - 1e-3);
        return c < 1.0 ? 1u : (uint32_t)c;
    };
    p.res = 0;
    p.gx = cells(lx); p.gy = cells(ly); p.gz = cells(lz);
    p.numCells = p.gx * p.gy * p.gz;
    p.inv_cell = T(inv);
    p.box_c = mk(T(0.5f * lx), T(0.5f * ly), T(0.5f * lz));
    p.box_b = p.box_c;
    derive_h(p, T(h));
}

// ---- SPH smoothing kernels: fluidkernel.cu:5-67 ----
template <class T> inline T poly6(const Params<T>& P, T r) {
    return (r >= P.h) ? T(0) : P.poly6 * pow_(fma_(-r, r, P.h2), T(3));
}
template <class T> inline T grad_poly6(const Params<T>& P, T r) {
    return (r >= P.h) ? T(0) : P.gradPoly6 * r * pow_(fma_(-r, r, P.h2), T(2));
}
template <class T> inline T grad_spiky(const Params<T>& P, T r) {
    return (r >= P.h) ? T(0) : P.gradSpiky * (P.h - r) * (P.h - r);
}
// fluidkernel.cu:35-38 with its precedence as written: the coefficient is
// multiplied by the comparison and only selects between the two branches.
template <class T> inline T cohesion_k(const Params<T>& P, T r) {
    if (r >= P.h) return T(0);
    const T sel = P.cohesion * T(r > P.halfh ? 1 : 0);
    const T hr3 = pow_(P.h - r, T(3));
    if (sel != T(0)) return hr3 * r * r * r;
    return T(2) * hr3 * r * r * r - P.h6 * T(0.0156f);
}
// fluidkernel.cu:45-67.  The leading 1.0 is a double literal: for the float
// build the difference is formed in double and rounded once to float.  The
// polynomial is evaluated with the multiply-adds fused the way the reference
// build fuses them (matched against its outputs in tests/golden/):
//   e1 = fma(35, c6, -(180 c4) h2); e2 = fma(378 c2, h4, e1);
//   e3 = fma(-420, h6, e2); f = fma(c3, e3, (315 c) h8) + 128 h9.
template <class T> inline T boundary_density(const Params<T>& P, T d) {
    if ((d > P.h) || (d < T(0))) return T(0);
    const T c = -d, c2 = c * c, c3 = c2 * c, c4 = c3 * c, c6 = c3 * c3;
    const T e1 = fma_(T(35), c6, -((T(180) * c4) * P.h2));
    const T e2 = fma_(T(378) * c2, P.h4, e1);
    const T e3 = fma_(T(-420), P.h6, e2);
    const T poly = fma_(c3, e3, (T(315) * c) * P.h8) + T(128) * P.h9;
    const T f = (T(0.0039062f) * P.invh9) * poly;
    return T(1.0 - double(f));
}

// ---- geometry: fluidutil.cu:85-112 ----
template <class T> inline T sdf_box(const Params<T>& P, V3<T> pos) {
    const V3<T> q = mk(std::fabs(pos.x - P.box_c.x) - P.box_b.x,
                       std::fabs(pos.y - P.box_c.y) - P.box_b.y,
                       std::fabs(pos.z - P.box_c.z) - P.box_b.z);
    // fminf/fmaxf semantics (a NaN operand yields the other operand)
    const T inner = std::fmin(std::fmax(q.x, std::fmax(q.y, q.z)), T(0));
    const V3<T> qp = mk(std::fmax(q.x, T(0)), std::fmax(q.y, T(0)), std::fmax(q.z, T(0)));
    return inner + sqrt_(dot(qp, qp));
}
// the sphere container: length(p - c) - r (fluidutil.cu:97-98), r the box's
// smallest half extent (0.5 in the unit cube, as there)
template <class T> inline T sdf_sphere(const Params<T>& P, V3<T> pos) {
    const V3<T> d = mk(pos.x - P.box_c.x, pos.y - P.box_c.y, pos.z - P.box_c.z);
    const T r = std::fmin(P.box_b.x, std::fmin(P.box_b.y, P.box_b.z));
    return sqrt_(dot(d, d)) - r;
}
template <class T> inline T sdf(const Params<T>& P, V3<T> pos) {
    return P.boundary == 1 ? sdf_sphere(P, pos) : sdf_box(P, pos);
}
template <class T> inline V3<T> normalize_(V3<T> v) {
    const T inv = T(1) / sqrt_(dot(v, v));
    return v * inv;
}
template <class T> inline V3<T> sdf_normal(const Params<T>& P, V3<T> p) {
    const T e = T(0.0001f);
    return normalize_(mk(sdf(P, mk(p.x + e, p.y, p.z)) - sdf(P, mk(p.x - e, p.y, p.z)),
                         sdf(P, mk(p.x, p.y + e, p.z)) - sdf(P, mk(p.x, p.y - e, p.z)),
                         sdf(P, mk(p.x, p.y, p.z + e)) - sdf(P, mk(p.x, p.y, p.z - e))));
}

// ---- spatial hash: hash.cu:10-27, fluidutil.cu:15-39 ----
template <class T> inline uint32_t hash_point(const Params<T>& P, V3<T> p) {
    // grid = floor(p * res) computed in the state precision, converted to int
    const int32_t gx = f2i_dev<T>(std::floor(p.x * P.inv_cell));
    const int32_t gy = f2i_dev<T>(std::floor(p.y * P.inv_cell));
    const int32_t gz = f2i_dev<T>(std::floor(p.z * P.inv_cell));
    const bool inside = gx >= 0 && gx < (int32_t)P.gx && gy >= 0 && gy < (int32_t)P.gy &&
                        gz >= 0 && gz < (int32_t)P.gz;
    return inside ? (uint32_t)gx + (uint32_t)gy * P.gx + (uint32_t)gz * P.gx * P.gy : NULL_HASH;
}

struct SimBase {
    virtual ~SimBase() {}
    virtual int precision() const = 0;
};

template <class T> struct Sim : SimBase {
    Params<T> P;
    bool isInit = false;
    std::vector<V3<T>> pos, vel, acc, nrm, fp, ft, fa, fv, colour, vint;   // vint: velocity before XSPH
    std::vector<T> rho, prs, cs, rho_sum;   // rho_sum: neighbour sum before the boundary term
    // Test scales (only with track_scales): per particle the sum over its
    // pairs of the magnitude of each pair's term in the pressure, viscosity
    // and tension forces and in the normal, scaled as the result is.  A sum
    // of cancelling terms has rounding error proportional to this, not to
    // the net value.  Off by default so that the timed oracle does no more
    // than the reference's arithmetic.
    bool track_scales = false;
    std::vector<T> sc_fp, sc_fv, sc_ft, sc_nrm;
    std::vector<uint32_t> hash_pre, hash, perm, cellOcc, cellStart, nbr;
    uint64_t substeps_done = 0;

    Sim() { ctor_defaults(P); }
    int precision() const override { return sizeof(T) == 4 ? 32 : 64; }

    // FluidSystem::init (fluidsystem.cu:196-265) array part.
    void alloc(uint32_t n) {
        P.numParticles = n;
        pos.assign(n, mk(T(0), T(0), T(0)));
        nrm.assign(n, mk(T(0), T(1), T(0)));
        vel.assign(n, mk(T(0), T(0), T(0)));
        acc.assign(n, mk(T(0), T(0), T(0)));
        fp.assign(n, mk(T(0), T(0), T(0)));
        ft = fa = fv = fp;
        colour = vint = fp;
        rho.assign(n, T(0)); prs.assign(n, T(0)); cs.assign(n, T(0)); rho_sum.assign(n, T(0));
        sc_fp.assign(n, T(0)); sc_fv.assign(n, T(0)); sc_ft.assign(n, T(0)); sc_nrm.assign(n, T(0));
        hash_pre.assign(n, 0); hash.assign(n, 0); perm.resize(n);
        for (uint32_t i = 0; i < n; ++i) perm[i] = i;
        nbr.assign(n, 0);
        cellOcc.assign(P.numCells, 0); cellStart.assign(P.numCells, 0);
        isInit = true;
    }
    void init(uint32_t n, uint32_t res) { init_defaults(P, n, res); alloc(n); }
    void resize_cells() { cellOcc.assign(P.numCells, 0); cellStart.assign(P.numCells, 0); }

    // FluidSystem::createFluidBlock (fluidsystem.cu:66-127).  Float arithmetic
    // as in the reference host code (cbrt of a float promotes to double there).
    int create_block(uint32_t first, uint32_t n, float mnx, float mny, float mnz, float mxx, float mxy, float mxz) {
        if ((uint64_t)first + n > P.numParticles) return 1;
        const float dx = mxx - mnx, dy = mxy - mny, dz = mxz - mnz;
        const float volume = dx * dy * dz;
        const float partVolume = volume / float(n);
        const float approx = std::cbrt(partVolume);   // float overload (cbrtf)
        const float rx = dx / approx + 0.5f, ry = dy / approx + 0.5f, rz = dz / approx + 0.5f;
        const float diam = std::min(std::min(dx / rx, dy / ry), dz / rz);
        set_mass(P, T(partVolume * float(P.restDensity)));
        set_psize(P, T(diam * 0.5f));
        uint32_t cnt = 0;
        float px, py, pz;
        for (px = mnx + 0.5f * diam; px <= mxx; px += diam)
            for (py = mny + 0.5f * diam; py <= mxy; py += diam)
                for (pz = mnz + 0.5f * diam; pz <= mxz; pz += diam)
                    if (cnt < n) { pos[first + cnt] = mk(T(px), T(py), T(pz)); cnt++; }
        return 0;
    }

    // ---- one substep: the body of the loop at fluidsystem.cu:301-398 ----
    void hash_and_sort() {
        const uint32_t n = P.numParticles;
        std::fill(cellOcc.begin(), cellOcc.end(), 0u);
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t h = hash_point(P, pos[i]);
            hash_pre[i] = h;
            if (h != NULL_HASH) cellOcc[h]++;
        }
        // thrust::sort_by_key on u32 keys is a stable radix sort: ties keep
        // their current order.  A stable counting sort gives the same order.
        std::vector<uint32_t> start(P.numCells + 1, 0);
        for (uint32_t c = 0; c < P.numCells; ++c) start[c + 1] = start[c] + cellOcc[c];
        uint32_t nullPos = start[P.numCells];
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t h = hash_pre[i];
            const uint32_t k = (h == NULL_HASH) ? nullPos++ : fill[h]++;
            perm[k] = i;
        }
        std::vector<V3<T>> p2(n), v2(n), a2(n);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t i = perm[k];
            hash[k] = hash_pre[i]; p2[k] = pos[i]; v2[k] = vel[i]; a2[k] = acc[i];
        }
        pos.swap(p2); vel.swap(v2); acc.swap(a2);
        // exclusive_scan(cellOcc) -> scatterAddress (fluidsystem.cu:316)
        for (uint32_t c = 0; c < P.numCells; ++c) cellStart[c] = start[c];
    }

    // Iterate the 27 neighbour cells of grid cell (bx,by,bz) in the
    // reference's order (fluidphysics.cu:30-53): x offset outermost, z
    // innermost, clipped at the grid edge; particles of a cell ascending.
    template <class F> inline void for_neighbours(uint32_t cell, F&& f) const {
        const uint32_t bx = cell % P.gx, by = (cell / P.gx) % P.gy, bz = cell / (P.gx * P.gy);
        for (int i = (bx == 0 ? 0 : -1); i <= (bx == P.gx - 1 ? 0 : 1); ++i)
            for (int j = (by == 0 ? 0 : -1); j <= (by == P.gy - 1 ? 0 : 1); ++j)
                for (int k = (bz == 0 ? 0 : -1); k <= (bz == P.gz - 1 ? 0 : 1); ++k) {
                    const uint32_t oc = (bx + i) + (by + j) * P.gx + (bz + k) * P.gx * P.gy;
                    const uint32_t s = cellStart[oc], e = s + cellOcc[oc];
                    for (uint32_t o = s; o < e; ++o) f(o);
                }
    }

    // computeDensity (fluidphysics.cu:8-84)
    void density() {
        const uint32_t n = P.numParticles;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            const uint32_t i = (uint32_t)ii;
            if (hash[i] == NULL_HASH) { rho[i] = T(0); prs[i] = T(0); cs[i] = T(0); nbr[i] = 0; continue; }
            const V3<T> pi = pos[i];
            T sum = T(0);
            uint32_t cnt = 0;
            for_neighbours(hash[i], [&](uint32_t o) {
                const V3<T> d = pi - pos[o];
                const T rr = dot(d, d);
                if (o != i && rr <= P.h2) { sum = fma_(P.mass, poly6(P, sqrt_(rr)), sum); cnt++; }
            });
            const T d = std::fabs(sdf(P, pi));
            T corr = sum;
            if (d < P.h) corr = fma_(P.restDensity, T(1.0f) - boundary_density(P, d), corr);
            rho_sum[i] = sum;
            rho[i] = (sum == T(0)) ? P.restDensity : corr;
            prs[i] = (corr == T(0)) ? T(0)
                   : (P.gasConstant * P.restDensity * P.invGamma) * (pow_(corr * P.invRestDensity, P.gamma) - T(1));
            cs[i] = P.gasConstant * pow_(corr * P.invRestDensity, P.gamma - T(1));
            nbr[i] = cnt;
        }
    }

    // computeNormals (fluidphysics.cu:154-210)
    void normals() {
        const uint32_t n = P.numParticles;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            const uint32_t i = (uint32_t)ii;
            if (hash[i] == NULL_HASH) { nrm[i] = mk(T(0), T(0), T(0)); continue; }
            V3<T> sum = mk(T(0), T(0), T(0));
            double mag = 0.0;
            for_neighbours(hash[i], [&](uint32_t o) {
                const V3<T> rv = pos[i] - pos[o];
                const T r2 = dot(rv, rv);
                if (o != i && rho[o] > P.eps && r2 <= P.h2 && r2 > P.eps) {
                    const T r = sqrt_(r2);
                    const V3<T> t = ((P.mass * grad_poly6(P, r)) * rv) / (rho[o] * r);
                    sum = sum + t;
                    if (track_scales) mag += vnorm(t);
                }
            });
            nrm[i] = P.h * sum;
            if (track_scales) sc_nrm[i] = T(std::fabs(double(P.h)) * mag);
        }
    }

    // computeAllForces (fluidphysics.cu:215-352)
    void forces() {
        const uint32_t n = P.numParticles;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            const uint32_t i = (uint32_t)ii;
            if (hash[i] == NULL_HASH) {
                fp[i] = ft[i] = fa[i] = fv[i] = mk(T(0), T(0), T(0));
                continue;
            }
            V3<T> ps = mk(T(0), T(0), T(0)), vs = ps, ts = ps;
            double mp = 0.0, mv = 0.0, mt = 0.0;   // test scales (track_scales)
            const V3<T> pi = pos[i], vi = vel[i], ni = nrm[i];
            const T ri = rho[i], pri = prs[i], csi = cs[i];
            for_neighbours(hash[i], [&](uint32_t o) {
                const V3<T> rv = pos[o] - pi;
                const T r2 = dot(rv, rv);
                if (o != i && rho[o] > P.eps && r2 <= P.h2 && r2 > P.eps) {
                    const T r = sqrt_(r2);
                    const T inv_r = T(1.0f) / r;
                    const V3<T> u = vi - vel[o];
                    const T ux = dot(u, -rv);
                    T Pi = T(0);
                    if (ux < T(0)) {
                        // fluidphysics.cu:279: 0.01 is a double literal
                        const T mu = T(double(P.h * ux) / (double(r2) + 0.01 * double(P.h2)));
                        Pi = (-P.viscosity * (csi + cs[o]) * mu) / (ri + rho[o]);
                    }
                    const T mid = prs[o] / (ri * ri) + pri / (rho[o] * rho[o]);
                    const V3<T> common = ((P.mass * grad_spiky(P, r)) * rv) * inv_r;
                    ps = fmaV(common, mid, ps);
                    vs = fmaV(common, mid + Pi, vs);
                    const V3<T> coh = ((-P.mass * P.mass * cohesion_k(P, r)) * rv) * inv_r;
                    const V3<T> curv = (-P.surfaceTension * P.mass) * (ni - nrm[o]);
                    const V3<T> tt = ((T(2.0f) * P.restDensity) * (coh + curv)) / (ri + ri);
                    ts = ts + tt;
                    if (track_scales) {
                        mp += vnorm(common * mid);
                        mv += vnorm(common * (mid + Pi));
                        // the curvature term takes the difference of two
                        // normals, each a cancelling sum with its own scale
                        mt += std::fabs(double(T(2.0f) * P.restDensity) / double(ri + ri)) *
                              (vnorm(coh) + std::fabs(double(P.surfaceTension) * double(P.mass)) *
                                                (double(sc_nrm[i]) + double(sc_nrm[o])));
                    }
                }
            });
            fp[i] = ps;
            fv[i] = P.viscosity * vs;
            ft[i] = P.surfaceTension * ts;
            if (track_scales) {
                sc_fp[i] = T(mp);
                sc_fv[i] = T(std::fabs(double(P.viscosity)) * mv);
                sc_ft[i] = T(std::fabs(double(P.surfaceTension)) * mt);
            }
            fa[i] = mk(T(0), T(0), T(0));
            const T z = -std::fmin(sdf(P, pi), T(0)) * T(0.25f) * P.invParticleSize;
            if (z < T(1)) {
                const V3<T> nb = sdf_normal(P, pi);
                const T denom = T(1.0f) / pow_(T(1) - z, T(3));
                fa[i] = (P.adhesion * ri * P.invRestDensity * denom) * nb;
            }
        }
    }

    // LeapfrogIntegratorOperator (fluidintegrator.cu:11-70) over all particles.
    void integrate() {
        const uint32_t n = P.numParticles;
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            const uint32_t i = (uint32_t)ii;
            V3<T> p = pos[i], v = vel[i];
            const V3<T> a = acc[i];
            // fluidsystem.cu:352-378: the force kernel writes viscosity into
            // the adhesion buffer and adhesion into the viscosity buffer, and
            // the integrator sums pressure, tension, "adhesion", "viscosity".
            const V3<T> force = ((fp[i] + ft[i]) + fv[i]) + fa[i];
            V3<T> an = fmaV(force, P.mass, P.gravity);
            T sq = dot(an, an);
            if (sq > P.accLimit2) an = an * (P.accLimit / sqrt_(sq));
            const V3<T> ha = T(0.5f) * a;
            p = mk(p.x + fma_(v.x, P.dt, ha.x * P.dtdt), p.y + fma_(v.y, P.dt, ha.y * P.dtdt),
                   p.z + fma_(v.z, P.dt, ha.z * P.dtdt));
            const V3<T> hs = T(0.5f) * (a + an);
            v = fmaV(hs, P.dt, v);
            sq = dot(v, v);
            if (sq > P.velLimit2) v = v * (P.velLimit / sqrt_(sq));
            const T d = sdf(P, p);
            if (d > -P.particleSize) {
                const V3<T> nb = sdf_normal(P, p);
                p = fmaV(-(d + P.particleSize), nb, p);
                const T k = (T(1.0f) + P.vdamp) * dot(nb, v);
                v = fmaV(-k, nb, v);
            }
            pos[i] = p; vel[i] = v; acc[i] = an; vint[i] = v;
        }
    }

    // correctVelocityXSPH (fluidphysics.cu:355-409) with Jacobi reads.
    void xsph() {
        const uint32_t n = P.numParticles;
        std::vector<V3<T>> vnew(vel);
#pragma omp parallel for schedule(static)
        for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
            const uint32_t i = (uint32_t)ii;
            if (hash[i] == NULL_HASH) continue;
            const V3<T> pi = pos[i];
            V3<T> sum = mk(T(0), T(0), T(0));
            for_neighbours(hash[i], [&](uint32_t o) {
                const V3<T> d = pi - pos[o];
                const T rr = dot(d, d);
                if (o != i && rr <= P.h2 && (rho[i] + rho[o]) > P.eps) {
                    const T r = sqrt_(rr);
                    const T coeff = poly6(P, r) * ((T(2.0f) * P.mass) / (rho[i] + rho[o]));
                    sum = fmaV(coeff, vel[o] - vel[i], sum);
                }
            });
            vnew[i] = fmaV(P.xsph, sum, vel[i]);
        }
        vel.swap(vnew);
    }

    void substep() {
        hash_and_sort();
        density();
        normals();
        forces();
        integrate();
        xsph();
        substeps_done++;
    }

    // DensityColourOperator (fluidutil.cu:67-80)
    void compute_colour() {
        for (uint32_t i = 0; i < P.numParticles; ++i) {
            const T ratio = rho[i] * P.invRestDensity;
            V3<T> c = mk(T(1), T(0), T(0));
            if (ratio < T(1)) c = mk(T(0), ratio, T(1) - ratio);
            else if (ratio < T(2)) c = mk(ratio - T(1), T(2) - ratio, T(0));
            colour[i] = c;
        }
    }
};

// Number of substeps FluidSystem::advance executes (fluidsystem.cu:294-301):
// a float loop variable accumulated by part_dt.  Returns -1 if the loop would
// never terminate (the accumulator stops growing before reaching full_dt).
int64_t substep_count(float full_dt, uint32_t substeps) {
    volatile float part = full_dt / float(substeps);
    volatile float dt = part;
    int64_t cnt = 0;
    while (dt <= full_dt) {
        cnt++;
        volatile float nx = dt + part;
        if (nx == dt) return -1;
        dt = nx;
        if (cnt > (int64_t)1 << 40) return -1;
    }
    return cnt;
}

}  // namespace

// ---------------------------------------------------------------------------
// C interface for ctypes (tests and bench only).
// ---------------------------------------------------------------------------
extern "C" {

enum {
    ORC_P_REST_DENSITY = 0, ORC_P_PARTICLE_SIZE, ORC_P_GAS_CONSTANT, ORC_P_XSPH, ORC_P_SURFACE_TENSION,
    ORC_P_VISCOSITY, ORC_P_ADHESION, ORC_P_VDAMP, ORC_P_GAMMA, ORC_P_MASS, ORC_P_DT
};
enum {
    ORC_F_POS = 0, ORC_F_VEL, ORC_F_ACC, ORC_F_NORMAL, ORC_F_FPRESSURE, ORC_F_FTENSION, ORC_F_FADHESION,
    ORC_F_FVISCOSITY, ORC_F_COLOUR, ORC_F_VEL_INT,        // vec3 fields
    ORC_F_DENSITY = 16, ORC_F_PRESSURE, ORC_F_SOUNDSPEED, ORC_F_RHOSUM,  // scalar fields
    ORC_F_SC_FPRESSURE, ORC_F_SC_FVISCOSITY, ORC_F_SC_FTENSION, ORC_F_SC_NORMAL,  // test scales
    ORC_F_HASH_PRE = 32, ORC_F_HASH, ORC_F_PERM, ORC_F_CELLSTART, ORC_F_CELLOCC, ORC_F_NBRCOUNT  // u32
};

void* orc_create(int precision) {
    if (precision == 64) return new Sim<double>();
    return new Sim<float>();
}
void orc_destroy(void* s) { delete (SimBase*)s; }
int orc_precision(void* s) { return ((SimBase*)s)->precision(); }

#define DISPATCH(s, ...) \
    do { SimBase* b__ = (SimBase*)(s); \
         if (b__->precision() == 32) { auto& S = *(Sim<float>*)b__; using T = float; (void)sizeof(T); __VA_ARGS__; } \
         else { auto& S = *(Sim<double>*)b__; using T = double; (void)sizeof(T); __VA_ARGS__; } } while (0)

int orc_init(void* s, uint32_t n, uint32_t res) { DISPATCH(s, S.init(n, res)); return 0; }
int orc_set_domain(void* s, float lx, float ly, float lz, float h) {
    if (!(h > 0.0f) || !(lx > 0.0f) || !(ly > 0.0f) || !(lz > 0.0f)) return 1;
    DISPATCH(s, { set_domain(S.P, lx, ly, lz, h); S.resize_cells(); });
    return 0;
}
// Boundary shape (0 box, 1 sphere); no reference setter: the reference
// always returns the box distance.
int orc_set_boundary(void* s, int shape) {
    if (shape != 0 && shape != 1) return 1;
    DISPATCH(s, S.P.boundary = shape);
    return 0;
}
int orc_set_param(void* s, int which, float v) {
    DISPATCH(s, {
        switch (which) {
            case ORC_P_REST_DENSITY: set_rest_density(S.P, T(v)); break;
            case ORC_P_PARTICLE_SIZE: set_psize(S.P, T(v)); break;
            case ORC_P_GAS_CONSTANT: S.P.gasConstant = T(v); break;
            case ORC_P_XSPH: S.P.xsph = T(v); break;
            case ORC_P_SURFACE_TENSION: S.P.surfaceTension = T(v); break;
            case ORC_P_VISCOSITY: S.P.viscosity = T(v); break;
            case ORC_P_ADHESION: S.P.adhesion = T(v); break;
            case ORC_P_VDAMP: S.P.vdamp = T(v); break;
            case ORC_P_GAMMA: set_gamma(S.P, T(v)); break;
            case ORC_P_MASS: set_mass(S.P, T(v)); break;
            case ORC_P_DT: set_dt(S.P, T(v)); break;
            default: return 1;
        }
    });
    return 0;
}
int orc_set_limits(void* s, float vl, float al) { DISPATCH(s, set_limits(S.P, T(vl), T(al))); return 0; }
int orc_set_gravity(void* s, float x, float y, float z) { DISPATCH(s, S.P.gravity = mk(T(x), T(y), T(z))); return 0; }
int orc_create_block(void* s, uint32_t first, uint32_t n, float a, float b, float c, float d, float e, float f) {
    int rc = 0;
    DISPATCH(s, rc = S.create_block(first, n, a, b, c, d, e, f));
    return rc;
}
// Copy positions/velocities (packed xyz float32) in, like setupFromData's copy.
int orc_set_state(void* s, const float* pos, const float* vel, uint32_t n) {
    int rc = 0;
    DISPATCH(s, {
        if (n != S.P.numParticles) rc = 1;
        else for (uint32_t i = 0; i < n; ++i) {
            S.pos[i] = mk(T(pos[3 * i]), T(pos[3 * i + 1]), T(pos[3 * i + 2]));
            if (vel) S.vel[i] = mk(T(vel[3 * i]), T(vel[3 * i + 1]), T(vel[3 * i + 2]));
        }
    });
    return rc;
}
// Full state in double (for seeding the FP64 twin with exactly the FP32 state).
int orc_set_state_f64(void* s, const double* pos, const double* vel, const double* acc, uint32_t n) {
    int rc = 0;
    DISPATCH(s, {
        if (n != S.P.numParticles) rc = 1;
        else for (uint32_t i = 0; i < n; ++i) {
            S.pos[i] = mk(T(pos[3 * i]), T(pos[3 * i + 1]), T(pos[3 * i + 2]));
            if (vel) S.vel[i] = mk(T(vel[3 * i]), T(vel[3 * i + 1]), T(vel[3 * i + 2]));
            if (acc) S.acc[i] = mk(T(acc[3 * i]), T(acc[3 * i + 1]), T(acc[3 * i + 2]));
        }
    });
    return rc;
}
int64_t orc_substep_count(float full_dt, uint32_t substeps) { return substep_count(full_dt, substeps); }
// FluidSystem::advance (fluidsystem.cu:273-399).  Returns substeps executed.
int64_t orc_advance(void* s, float full_dt, uint32_t substeps) {
    int64_t cnt = substep_count(full_dt, substeps);
    if (cnt < 0) return -1;
    DISPATCH(s, {
        if (!S.isInit) return 0;
        set_dt(S.P, T(full_dt / float(substeps)));
        for (int64_t k = 0; k < cnt; ++k) S.substep();
    });
    return cnt;
}
// Individual stages, for per-pass parity tests.
int orc_stage(void* s, int which) {
    DISPATCH(s, {
        switch (which) {
            case 0: S.hash_and_sort(); break;
            case 1: S.density(); break;
            case 2: S.normals(); break;
            case 3: S.forces(); break;
            case 4: S.integrate(); break;
            case 5: S.xsph(); break;
            case 6: S.compute_colour(); break;
            default: return 1;
        }
    });
    return 0;
}
uint32_t orc_num_particles(void* s) { uint32_t n = 0; DISPATCH(s, n = S.P.numParticles); return n; }
uint32_t orc_num_cells(void* s) { uint32_t n = 0; DISPATCH(s, n = S.P.numCells); return n; }
// Derived parameters as doubles, in a fixed order (see libfluid_gb300 tests).
int orc_get_params(void* s, double* out, int cap) {
    int k = 0;
    DISPATCH(s, {
        const auto& p = S.P;
        const double v[] = {double(p.gx), double(p.gy), double(p.gz), double(p.inv_cell), double(p.h), double(p.h2),
                            double(p.poly6), double(p.gradPoly6), double(p.gradSpiky), double(p.cohesion),
                            double(p.invh9), double(p.restDensity), double(p.gasConstant), double(p.gamma),
                            double(p.mass), double(p.particleSize), double(p.dt), double(p.xsph),
                            double(p.surfaceTension), double(p.viscosity), double(p.adhesion), double(p.vdamp),
                            double(p.velLimit), double(p.accLimit), double(p.gravity.x), double(p.gravity.y),
                            double(p.gravity.z), double(p.eps)};
        for (; k < cap && k < (int)(sizeof(v) / sizeof(v[0])); ++k) out[k] = v[k];
    });
    return k;
}
// Field readback.  vec3 fields -> 3*n values; scalars -> n; u32 -> n (or cells).
// Floating fields are written as double (out_f64) or float (out_f32).
int orc_get(void* s, int field, float* out_f32, double* out_f64, uint32_t* out_u32, uint64_t cap) {
    int rc = 0;
    DISPATCH(s, {
        const uint32_t n = S.P.numParticles;
        const std::vector<V3<T>>* v3 = nullptr;
        const std::vector<T>* sc = nullptr;
        const std::vector<uint32_t>* u = nullptr;
        switch (field) {
            case ORC_F_POS: v3 = &S.pos; break;
            case ORC_F_VEL: v3 = &S.vel; break;
            case ORC_F_ACC: v3 = &S.acc; break;
            case ORC_F_NORMAL: v3 = &S.nrm; break;
            case ORC_F_FPRESSURE: v3 = &S.fp; break;
            case ORC_F_FTENSION: v3 = &S.ft; break;
            case ORC_F_FADHESION: v3 = &S.fa; break;
            case ORC_F_FVISCOSITY: v3 = &S.fv; break;
            case ORC_F_COLOUR: v3 = &S.colour; break;
            case ORC_F_VEL_INT: v3 = &S.vint; break;
            case ORC_F_DENSITY: sc = &S.rho; break;
            case ORC_F_PRESSURE: sc = &S.prs; break;
            case ORC_F_SOUNDSPEED: sc = &S.cs; break;
            case ORC_F_RHOSUM: sc = &S.rho_sum; break;
            case ORC_F_SC_FPRESSURE: sc = &S.sc_fp; break;
            case ORC_F_SC_FVISCOSITY: sc = &S.sc_fv; break;
            case ORC_F_SC_FTENSION: sc = &S.sc_ft; break;
            case ORC_F_SC_NORMAL: sc = &S.sc_nrm; break;
            case ORC_F_HASH_PRE: u = &S.hash_pre; break;
            case ORC_F_HASH: u = &S.hash; break;
            case ORC_F_PERM: u = &S.perm; break;
            case ORC_F_CELLSTART: u = &S.cellStart; break;
            case ORC_F_CELLOCC: u = &S.cellOcc; break;
            case ORC_F_NBRCOUNT: u = &S.nbr; break;
            default: rc = 1;
        }
        if (v3) {
            if (cap < 3ull * n) rc = 2;
            else for (uint32_t i = 0; i < n; ++i) {
                const V3<T> q = (*v3)[i];
                if (out_f64) { out_f64[3 * i] = q.x; out_f64[3 * i + 1] = q.y; out_f64[3 * i + 2] = q.z; }
                if (out_f32) { out_f32[3 * i] = float(q.x); out_f32[3 * i + 1] = float(q.y); out_f32[3 * i + 2] = float(q.z); }
            }
        } else if (sc) {
            if (cap < n) rc = 2;
            else for (uint32_t i = 0; i < n; ++i) {
                if (out_f64) out_f64[i] = (*sc)[i];
                if (out_f32) out_f32[i] = float((*sc)[i]);
            }
        } else if (u) {
            if (cap < u->size() || !out_u32) rc = 2;
            else std::memcpy(out_u32, u->data(), u->size() * sizeof(uint32_t));
        }
    });
    return rc;
}
// Test scales of the force and normal sums (Sim::track_scales).
int orc_track_scales(void* s, int on) { DISPATCH(s, S.track_scales = on != 0); return 0; }
int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"
