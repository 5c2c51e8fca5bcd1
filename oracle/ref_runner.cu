// Runs the reference's own device code (oracle/_ref/libfluid_ref.cubin, built
// from NCCA/libfluid's cudasrc by oracle/ref_build.sh) on the GPU.
//
// TEST INFRASTRUCTURE ONLY: it produces the golden vectors that pin the oracle
// (tests/golden/) and times the reference's CUDA step for comparison.
//
// The host orchestration restates FluidSystem::advance's substep
// (fluidsystem.cu:301-398) step for step: fill cellOcc; transform with
// PointHashOperator; thrust::sort_by_key(hash, zip(P,V,A)); exclusive_scan;
// reduce(max); blockSize = 32*ceil(maxOcc/32); computeDensity, sync;
// computeNormals, sync; computeAllForces (buffers in the reference's argument
// order), sync; for_each(LeapfrogIntegratorOperator); correctVelocityXSPH,
// sync.  An index array rides along in the sort to expose the permutation.
//
// usage: ref_runner <dir with libfluid_ref.cubin> run  <in.bin> <out.bin>
//        ref_runner <dir> time <in.bin> <warmup> <steps>
// in.bin:  u32 magic 0x53504831, n, res, substeps; f32 part_dt; 16 f32
//          parameters (see read_input); P[3n] f32; V[3n] f32
// out.bin: u32 n, cells; then the fields listed in dump().
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#define CK(x)                                                                      \
    do {                                                                           \
        cudaError_t e_ = (x);                                                      \
        if (e_ != cudaSuccess) {                                                   \
            fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            exit(3);                                                               \
        }                                                                          \
    } while (0)
#define CKD(x)                                                                     \
    do {                                                                           \
        CUresult r_ = (x);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                  \
            const char* s_ = nullptr;                                              \
            cuGetErrorString(r_, &s_);                                             \
            fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, s_ ? s_ : "?"); \
            exit(3);                                                               \
        }                                                                          \
    } while (0)

struct Input {
    uint32_t n = 0, res = 0, substeps = 1;
    float dt = 0.f;
    float rest_density, gas_constant, gamma, mass, particle_size, xsph, surface_tension, viscosity, adhesion,
        vdamp, vel_limit, acc_limit, gx, gy, gz, unused;
    std::vector<float> P, V;
};

static Input read_input(const char* path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    uint32_t hdr[4];
    f.read((char*)hdr, sizeof(hdr));
    if (hdr[0] != 0x53504831u) { fprintf(stderr, "bad magic\n"); exit(2); }
    Input in;
    in.n = hdr[1]; in.res = hdr[2]; in.substeps = hdr[3];
    f.read((char*)&in.dt, 4);
    float p[16];
    f.read((char*)p, sizeof(p));
    in.rest_density = p[0]; in.gas_constant = p[1]; in.gamma = p[2]; in.mass = p[3]; in.particle_size = p[4];
    in.xsph = p[5]; in.surface_tension = p[6]; in.viscosity = p[7]; in.adhesion = p[8]; in.vdamp = p[9];
    in.vel_limit = p[10]; in.acc_limit = p[11]; in.gx = p[12]; in.gy = p[13]; in.gz = p[14];
    in.P.resize(3ull * in.n);
    in.V.resize(3ull * in.n);
    f.read((char*)in.P.data(), in.P.size() * 4);
    f.read((char*)in.V.data(), in.V.size() * 4);
    if (!f) { fprintf(stderr, "short input\n"); exit(2); }
    return in;
}

// FluidParams derivations (fluidparams.cu:51-213), in ref_pack_params' order.
static void derive(const Input& in, std::vector<float>& v, std::vector<uint32_t>& u) {
    const float pi = 3.141592654f;
    const float h = 1.0f / float(in.res);
    u = {in.res, in.res * in.res, in.res * in.res * in.res, in.n};
    v.assign(50, 0.f);
    v[0] = in.rest_density;
    v[1] = in.rest_density == 0.f ? 1.f : 1.f / in.rest_density;
    v[2] = in.gas_constant;
    v[3] = in.gamma;
    v[4] = in.gamma == 0.f ? 1.f : 1.f / in.gamma;
    v[5] = in.mass; v[6] = in.mass * in.mass; v[7] = 1.f / in.mass;
    v[8] = in.particle_size; v[9] = 1.f / in.particle_size;
    v[10] = in.dt; v[11] = in.dt * in.dt;
    const float h2 = h * h, h3 = h * h * h, h4 = h * h * h * h, h5 = h3 * h2, h6 = h3 * h3, h8 = h5 * h3,
                h9 = h6 * h3;
    v[12] = h; v[13] = 0.5f * h; v[14] = h2; v[15] = h3; v[16] = h4; v[17] = h5; v[18] = h6; v[19] = h8;
    v[20] = h9; v[21] = 1.f / h; v[22] = 1.f / h2; v[23] = 1.f / h3; v[24] = 1.f / h6; v[25] = 1.f / (h6 * h3);
    v[26] = 1.f - h;
    v[27] = in.xsph; v[28] = in.surface_tension; v[29] = in.viscosity; v[30] = in.adhesion;
    v[31] = in.vel_limit; v[32] = in.acc_limit; v[33] = in.vel_limit * in.vel_limit;
    v[34] = in.acc_limit * in.acc_limit; v[35] = in.vdamp;
    v[36] = 2600.f; v[37] = 2600.f * 2600.f; v[38] = 1.f / 2600.f;   // DEFAULT_BOUNDARY_DENSITY
    v[39] = in.gx; v[40] = in.gy; v[41] = in.gz;
    v[42] = 315.0f / (64.0f * pi * powf(h, 9.0f));
    v[43] = -945.0f / (32.0f * pi * powf(h, 9.0f));
    v[44] = -945.0f / (32.0f * pi * powf(h, 9.0f));
    v[45] = 15.0f / (pi * powf(h, 6.0f));
    v[46] = -45.0f / (pi * powf(h, 6.0f));
    v[47] = 45.0f / (pi * powf(h, 6.0f));
    v[48] = 32.0f / (pi * powf(h, 9.0f));
    v[49] = FLT_MIN;
}

struct Ref {
    CUmodule mod;
    CUfunction density, normals, forces, xsph, hash, integrate, colour, count, pack, layout;
    CUdeviceptr params;
    size_t params_size;
};

static Ref load(const std::string& dir) {
    Ref r{};
    CKD(cuInit(0));
    CK(cudaFree(0));   // make the runtime's primary context current
    CKD(cuModuleLoad(&r.mod, (dir + "/libfluid_ref.cubin").c_str()));
    std::ifstream k(dir + "/kernels.txt");
    std::string name;
    while (k >> name) {
        CUfunction f;
        CKD(cuModuleGetFunction(&f, r.mod, name.c_str()));
        if (name.find("computeDensity") != std::string::npos) r.density = f;
        else if (name.find("computeNormals") != std::string::npos) r.normals = f;
        else if (name.find("computeAllForces") != std::string::npos) r.forces = f;
        else if (name.find("correctVelocityXSPH") != std::string::npos) r.xsph = f;
    }
    if (!r.density || !r.normals || !r.forces || !r.xsph) { fprintf(stderr, "kernels.txt incomplete\n"); exit(2); }
    CKD(cuModuleGetFunction(&r.hash, r.mod, "ref_hash"));
    CKD(cuModuleGetFunction(&r.integrate, r.mod, "ref_integrate"));
    CKD(cuModuleGetFunction(&r.colour, r.mod, "ref_colour"));
    CKD(cuModuleGetFunction(&r.count, r.mod, "ref_count_neighbours"));
    CKD(cuModuleGetFunction(&r.pack, r.mod, "ref_pack_params"));
    CKD(cuModuleGetFunction(&r.layout, r.mod, "ref_layout"));
    CKD(cuModuleGetGlobal(&r.params, &r.params_size, r.mod, "params"));
    return r;
}

static void launch(CUfunction f, dim3 g, dim3 b, void** args) {
    CKD(cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, 0, 0, args, nullptr));
}

struct Sim {
    uint32_t n, res, cells;
    float3 *P, *V, *A, *N, *fp, *ft, *fa, *fv, *colour, *vint;   // vint: velocity before XSPH
    float *rho, *prs, *cs;
    uint32_t *hash, *occ, *scatter, *idx, *nbr;
};

static void alloc(Sim& s) {
    float3** v3[] = {&s.P, &s.V, &s.A, &s.N, &s.fp, &s.ft, &s.fa, &s.fv, &s.colour, &s.vint};
    for (auto p : v3) { CK(cudaMalloc((void**)p, (size_t)s.n * sizeof(float3))); CK(cudaMemset(*p, 0, (size_t)s.n * sizeof(float3))); }
    float** sc[] = {&s.rho, &s.prs, &s.cs};
    for (auto p : sc) { CK(cudaMalloc((void**)p, (size_t)s.n * 4)); CK(cudaMemset(*p, 0, (size_t)s.n * 4)); }
    CK(cudaMalloc((void**)&s.hash, (size_t)s.n * 4));
    CK(cudaMalloc((void**)&s.idx, (size_t)s.n * 4));
    CK(cudaMalloc((void**)&s.nbr, (size_t)s.n * 4));
    CK(cudaMalloc((void**)&s.occ, (size_t)s.cells * 4));
    CK(cudaMalloc((void**)&s.scatter, (size_t)s.cells * 4));
    // m_Normals starts at (0,1,0) (fluidsystem.cu:239)
    std::vector<float3> up(s.n, make_float3(0.f, 1.f, 0.f));
    CK(cudaMemcpy(s.N, up.data(), (size_t)s.n * sizeof(float3), cudaMemcpyHostToDevice));
}

// One substep; returns the block size used (0 if nothing was launched).
// track_perm adds the sort permutation (an index payload) for the parity
// dumps; timed runs sort exactly fluidsystem.cu:309-313's P, V, A payload.
static uint32_t substep(const Ref& r, Sim& s, bool count_nbr, bool track_perm) {
    const uint32_t n = s.n;
    CKD(cuMemsetD32((CUdeviceptr)s.occ, 0, s.cells));
    {
        void* op = s.occ;          // PointHashOperator{cellOcc}, passed by value
        void* args[] = {&op, &s.P, &s.hash, (void*)&n};
        launch(r.hash, dim3((n + 255) / 256), dim3(256), args);
    }
    if (track_perm) {
        thrust::sequence(thrust::device, thrust::device_ptr<uint32_t>(s.idx), thrust::device_ptr<uint32_t>(s.idx) + n);
        thrust::sort_by_key(thrust::device, thrust::device_ptr<uint32_t>(s.hash),
                            thrust::device_ptr<uint32_t>(s.hash) + n,
                            thrust::make_zip_iterator(thrust::make_tuple(thrust::device_ptr<float3>(s.P),
                                                                         thrust::device_ptr<float3>(s.V),
                                                                         thrust::device_ptr<float3>(s.A),
                                                                         thrust::device_ptr<uint32_t>(s.idx))));
    } else {
        thrust::sort_by_key(thrust::device, thrust::device_ptr<uint32_t>(s.hash),
                            thrust::device_ptr<uint32_t>(s.hash) + n,
                            thrust::make_zip_iterator(thrust::make_tuple(thrust::device_ptr<float3>(s.P),
                                                                         thrust::device_ptr<float3>(s.V),
                                                                         thrust::device_ptr<float3>(s.A))));
    }
    thrust::exclusive_scan(thrust::device, thrust::device_ptr<uint32_t>(s.occ),
                           thrust::device_ptr<uint32_t>(s.occ) + s.cells, thrust::device_ptr<uint32_t>(s.scatter));
    const uint32_t maxOcc = thrust::reduce(thrust::device, thrust::device_ptr<uint32_t>(s.occ),
                                           thrust::device_ptr<uint32_t>(s.occ) + s.cells, 0u,
                                           thrust::maximum<uint32_t>());
    const uint32_t bs = 32 * (uint32_t)ceil(maxOcc / 32.0f);
    if (bs == 0) return 0;
    if (bs > 1024) { fprintf(stderr, "cell occupancy %u exceeds one block; the reference cannot launch\n", maxOcc); exit(4); }
    const dim3 grid(s.res, s.res, s.res), block(bs);
    {
        void* args[] = {&s.prs, &s.cs, &s.rho, &s.P, &s.occ, &s.scatter};
        launch(r.density, grid, block, args);
        CK(cudaDeviceSynchronize());
    }
    if (count_nbr) {
        void* args[] = {&s.P, &s.occ, &s.scatter, &s.nbr};
        launch(r.count, grid, block, args);
        CK(cudaDeviceSynchronize());
    }
    {
        void* args[] = {&s.N, &s.rho, &s.P, &s.occ, &s.scatter};
        launch(r.normals, grid, block, args);
        CK(cudaDeviceSynchronize());
    }
    {
        // kernel signature order: pressure, tension, adhesion, viscosity
        void* args[] = {&s.fp, &s.ft, &s.fa, &s.fv, &s.cs, &s.prs, &s.rho, &s.P, &s.N, &s.V, &s.occ, &s.scatter};
        launch(r.forces, grid, block, args);
        CK(cudaDeviceSynchronize());
    }
    {
        // for_each zip order P,V,A,m_Pressure,m_Tension,m_Adhesion,m_Viscosity; after the
        // swapped launch arguments m_Adhesion holds viscosity and m_Viscosity adhesion
        char op = 0;
        void* args[] = {&op, &s.P, &s.V, &s.A, &s.fp, &s.ft, &s.fv, &s.fa, (void*)&n};
        launch(r.integrate, dim3((n + 255) / 256), dim3(256), args);
    }
    if (count_nbr) CK(cudaMemcpy(s.vint, s.V, (size_t)n * sizeof(float3), cudaMemcpyDeviceToDevice));
    {
        void* args[] = {&s.V, &s.rho, &s.P, &s.occ, &s.scatter};
        launch(r.xsph, grid, block, args);
        CK(cudaDeviceSynchronize());
    }
    return bs;
}

template <class T>
static void put(std::ofstream& f, const T* dev, size_t count) {
    std::vector<T> h(count);
    CK(cudaMemcpy(h.data(), dev, count * sizeof(T), cudaMemcpyDeviceToHost));
    f.write((const char*)h.data(), count * sizeof(T));
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: ref_runner <dir> run <in> <out> | time <in> <warmup> <steps>\n");
        return 1;
    }
    const std::string dir = argv[1], mode = argv[2];
    Input in = read_input(argv[3]);
    Ref r = load(dir);
    {
        uint32_t* d = nullptr;
        CK(cudaMalloc((void**)&d, 64));
        void* args[] = {&d};
        launch(r.layout, dim3(1), dim3(1), args);
        uint32_t lay[5];
        CK(cudaMemcpy(lay, d, sizeof(lay), cudaMemcpyDeviceToHost));
        if (lay[0] != r.params_size || lay[1] != sizeof(void*) || lay[2] != 1 || lay[3] != 1 || lay[4] != 12) {
            fprintf(stderr, "unexpected layout %u %u %u %u %u\n", lay[0], lay[1], lay[2], lay[3], lay[4]);
            return 2;
        }
        std::vector<float> v;
        std::vector<uint32_t> u;
        derive(in, v, u);
        float* dv = nullptr;
        uint32_t* du = nullptr;
        void* staging = nullptr;
        CK(cudaMalloc((void**)&dv, v.size() * 4));
        CK(cudaMalloc((void**)&du, u.size() * 4));
        CK(cudaMalloc(&staging, r.params_size));
        CK(cudaMemcpy(dv, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(du, u.data(), u.size() * 4, cudaMemcpyHostToDevice));
        void* pargs[] = {&dv, &du, &staging};
        launch(r.pack, dim3(1), dim3(1), pargs);
        CK(cudaDeviceSynchronize());
        CKD(cuMemcpyDtoD(r.params, (CUdeviceptr)staging, r.params_size));
        CK(cudaDeviceSynchronize());
    }
    Sim s{};
    s.n = in.n; s.res = in.res; s.cells = in.res * in.res * in.res;
    alloc(s);
    CK(cudaMemcpy(s.P, in.P.data(), in.P.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.V, in.V.data(), in.V.size() * 4, cudaMemcpyHostToDevice));
    if (mode == "run") {
        if (argc < 5) return 1;
        uint32_t bs = 0;
        for (uint32_t k = 0; k < in.substeps; ++k) bs = substep(r, s, k + 1 == in.substeps, true);
        char op = 0;
        void* cargs[] = {&op, &s.rho, &s.colour, &s.n};
        launch(r.colour, dim3((s.n + 255) / 256), dim3(256), cargs);
        CK(cudaDeviceSynchronize());
        std::ofstream f(argv[4], std::ios::binary);
        const uint32_t hdr[3] = {s.n, s.cells, bs};
        f.write((const char*)hdr, sizeof(hdr));
        put(f, s.hash, s.n); put(f, s.idx, s.n); put(f, s.occ, s.cells); put(f, s.scatter, s.cells);
        put(f, s.nbr, s.n); put(f, s.rho, s.n); put(f, s.prs, s.n); put(f, s.cs, s.n);
        float3* v3[] = {s.N, s.fp, s.ft, s.fa, s.fv, s.P, s.V, s.A, s.colour, s.vint};
        for (auto p : v3) put(f, (const float*)p, 3ull * s.n);
        printf("{\"ok\": true, \"block\": %u}\n", bs);
        return 0;
    }
    if (mode == "time") {
        if (argc < 6) return 1;
        const int warm = atoi(argv[4]), steps = atoi(argv[5]);
        for (int k = 0; k < warm; ++k) substep(r, s, false, false);
        CK(cudaDeviceSynchronize());
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, 0));
        uint32_t bs = 0;
        for (int k = 0; k < steps; ++k) bs = substep(r, s, false, false);
        CK(cudaEventRecord(e1, 0));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        printf("{\"ms\": %.6f, \"steps\": %d, \"n\": %u, \"block\": %u}\n", ms, steps, s.n, bs);
        return 0;
    }
    return 1;
}
