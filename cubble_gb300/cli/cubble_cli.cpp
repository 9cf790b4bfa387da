// cubble-cli: drop-in for the reference's executable (`cubble-cli
// input_parameters.json`, src/main.cpp:22-25 -> cubble::run,
// src/simulator.cu:1161-1186). Host C++ over the C ABI of libcubble_gb300:
//   init()      src/simulator.cu:527-956  input JSON, lattice + cuRAND MTGP32
//               draws, first search, Euler start, stabilisation rounds, box
//               rescale to the target gas fraction, energy-converged
//               stabilisation
//   simulate()  src/simulator.cu:958-1158 the step loop with results.dat rows
//               and the stdout table at each scaled time unit, CSV snapshots
//               written by an IO thread, stop on numEnd / largest radius
//   saveSnapshot src/simulator.cu:387-512
// The step loop runs whole stretches between output times as one graph
// launch (cb_integrate_until checks the reference's stop and output
// conditions on the device after every step).
//
// Extensions (not in the reference): the optional input key
// "gb300": {"precision": "fp64" | "mixed" | "fp64_ff", "graph": 0 | 1, "shear": v} (v:
// maximum speed of a linear shear flow replacing the flow box), and the flags
//   --precision fp64|mixed|fp64_ff   --no-graph
//   --checkpoint FILE        write the full state at every printed time unit
//   --resume FILE            continue a run from such a checkpoint
//   --max-steps N            stop after N integration steps (testing)
//   --output-digits N        significant digits of results.dat and the
//                            snapshots (default 6, the reference's default
//                            stream precision; 17 round-trips a double)
//   --array FILE             expand an array.params file
//                            (scripts/triton/array_job.py:54-75) into one
//                            run per parameter set, each in run_<k>/.
//   --profile-range          the reference's PROFILE build option as a flag:
//                            the profiler's capture range (cudaProfilerStart /
//                            Stop) opens when the step loop starts and closes
//                            after 1000 steps within one time unit or after
//                            the loop's first printed time unit
//                            (src/util.cuh:38-52, src/simulator.cu:993,
//                            :1009)
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>
#include <curand.h>
#include <nvtx3/nvToolsExt.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cubble_gb300.h"
#include "json.hpp"

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993;

// Significant digits of the output files (--output-digits).
int g_output_digits = 6;
// --profile-range: open the profiler's capture range over the step loop.
bool g_profile_range = false;

void check(int rc, const char *what) {
    if (rc != CB_OK)
        throw std::runtime_error(std::string(what) + " failed: " + cb_last_error());
}

void check_curand(curandStatus_t st, const char *what) {
    if (st != CURAND_STATUS_SUCCESS)
        throw std::runtime_error(std::string(what) + " failed (cuRAND status " +
                                 std::to_string((int)st) + ")");
}

void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

struct Vec3 {
    double x = 0.0, y = 0.0, z = 0.0;
};

Vec3 vec_of(const cbj::Value &v) {
    Vec3 r;
    r.x = v["x"].number();
    r.y = v["y"].number();
    r.z = v["z"].number();
    return r;
}

// Everything simulate() needs besides the device state (HostData and the
// parts of Constants the host reads, src/data_definitions.h:183-269).
struct Run {
    cb_config cfg{};
    cb_context *ctx = nullptr;
    double avg_rad = 0.0, phi = 0.0, time_scaling = 0.0;
    double energy1 = 0.0, energy2 = 0.0;
    double snapshot_frequency = 0.0, max_delta_energy = 0.0;
    int32_t min_num_bubbles = 0;
    int32_t stabilization_steps = 0;
    uint32_t times_printed = 0, num_snapshots = 0;
    bool add_flow = false;
    Vec3 rel_dim;
    std::string snapshot_name;
    int64_t max_steps = -1;
    std::string checkpoint;
    // snapshot bookkeeping (previous positions by bubble index)
    std::vector<double> prev_x, prev_y, prev_z;
    std::thread io;
};

double box_volume(const cb_config &c) {
    const double ix = c.tfr[0] - c.lbb[0], iy = c.tfr[1] - c.lbb[1], iz = c.tfr[2] - c.lbb[2];
    return c.dimensionality == 3 ? ix * iy * iz : ix * iy;
}

double energy(Run &r) {
    double e = 0.0;
    check(cb_energy(r.ctx, &e), "cb_energy");
    return e;
}

cb_report report(Run &r) {
    cb_report rep{};
    check(cb_get_report(r.ctx, &rep), "cb_get_report");
    return rep;
}

// stabilize(), src/simulator.cu:338-360: n steps without gas exchange, flow
// or path, energies before and after.
void stabilize(Run &r, int32_t n) {
    nvtxRangePushA("Stabilization");
    r.energy1 = energy(r);
    check(cb_set_options(r.ctx, 0, 0, 0), "cb_set_options");
    cb_report rep{};
    check(cb_integrate(r.ctx, n, &rep), "cb_integrate");
    r.energy2 = energy(r);
    nvtxRangePop();
}

// printRelevantInfoOfCurrentDevice, src/util.cuh:222-251
void print_device() {
    int dev = 0;
    cudaDeviceProp p{};
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess)
        return;
    std::printf("\n---------------Properties of current device----------------");
    std::printf("\n\tName: %s\n\tCompute capability: %d.%d", p.name, p.major, p.minor);
    std::printf("\n\tMultiprocessors: %d\n\tGlobal memory: %zu MiB", p.multiProcessorCount,
                (size_t)(p.totalGlobalMem >> 20));
    std::printf("\n\tShared memory per block: %zu KiB\n\tL2 cache: %d MiB",
                (size_t)(p.sharedMemPerBlockOptin >> 10), p.l2CacheSize >> 20);
    std::printf("\n-----------------------------------------------------------\n");
}

void set_time(Run &r, uint64_t ti, double tf) {
    const cb_report rep = report(r);
    check(cb_set_time(r.ctx, rep.time_step, ti, tf), "cb_set_time");
}

// ------------------------------------------------------------------ init()
int precision_code(const std::string &name) {
    if (name == "mixed") return CB_PRECISION_MIXED;
    if (name == "fp64_ff") return CB_PRECISION_FP64_FF;
    return CB_PRECISION_FP64;
}
const char *precision_name(int p) {
    return p == CB_PRECISION_MIXED ? "mixed" : p == CB_PRECISION_FP64_FF ? "fp64_ff" : "fp64";
}

void init(Run &r, const cbj::Value &in, int precision_override, int graph_override) {
    const cbj::Value &constants = in["constants"], &bubbles = in["bubbles"], &box = in["box"];
    const cbj::Value &wall = box["wall"], &flow = in["flow"];
    r.stabilization_steps = (int32_t)in["stabilization"]["steps"].number();
    r.max_delta_energy = in["stabilization"]["maxDeltaEnergy"].number();
    r.avg_rad = bubbles["radius"]["mean"].number();
    r.min_num_bubbles = (int32_t)bubbles["numEnd"].number();
    cb_config &c = r.cfg;
    std::memset(&c, 0, sizeof(c));
    c.skin_radius = 0.3 * r.avg_rad;
    const double mu = constants["mu"]["value"].number();
    r.phi = constants["phi"]["value"].number();
    c.min_rad = 0.1 * r.avg_rad;
    c.f0_per_mu0 = (double)(float)constants["sigma"]["value"].number() * r.avg_rad / mu;
    c.k_parameter = constants["K"]["value"].number();
    c.kappa = constants["kappa"]["value"].number();
    r.time_scaling = c.k_parameter / (r.avg_rad * r.avg_rad);
    r.add_flow = 1 == flow["impose"].integer();
    const Vec3 flbb = vec_of(flow["lbb"]), ftfr = vec_of(flow["tfr"]);
    const Vec3 fvel = vec_of(flow["velocity"]);
    c.flow_lbb[0] = flbb.x, c.flow_lbb[1] = flbb.y, c.flow_lbb[2] = flbb.z;
    c.flow_tfr[0] = ftfr.x, c.flow_tfr[1] = ftfr.y, c.flow_tfr[2] = ftfr.z;
    c.flow_vel[0] = fvel.x * c.f0_per_mu0;
    c.flow_vel[1] = fvel.y * c.f0_per_mu0;
    c.flow_vel[2] = fvel.z * c.f0_per_mu0;
    c.error_tolerance = in["errorTolerance"]["value"].number();
    r.snapshot_frequency = in["snapShot"]["frequency"].number();
    r.snapshot_name = in["snapShot"]["filename"].string();
    c.wall_drag = wall["drag"].number();
    c.wall[0] = 1 == wall["x"].integer();
    c.wall[1] = 1 == wall["y"].integer();
    c.wall[2] = 1 == wall["z"].integer();
    c.dimensionality = box["dimensionality"].integer();
    if (c.dimensionality != 2 && c.dimensionality != 3)
        throw std::runtime_error("box.dimensionality must be 2 or 3");

    // box and bubble count from numStart and the relative dimensions
    // (src/simulator.cu:576-602, in the reference's float arithmetic)
    const float d = 2 * (float)r.avg_rad;
    float n = (float)bubbles["numStart"].number();
    r.rel_dim = vec_of(box["relativeDimensions"]);
    int32_t bpd[3] = {1, 1, 1};
    int32_t count = 0;
    if (c.dimensionality == 3) {
        n = std::cbrt(n);
        const float a = (float)std::cbrt(r.rel_dim.x / r.rel_dim.y);
        const float b = (float)std::cbrt(r.rel_dim.x / r.rel_dim.z);
        const float cc = (float)std::cbrt(r.rel_dim.y / r.rel_dim.z);
        bpd[0] = (int32_t)std::ceil(n * a * b);
        bpd[1] = (int32_t)std::ceil(n * cc / a);
        bpd[2] = (int32_t)std::ceil(n / (b * cc));
        count = bpd[0] * bpd[1] * bpd[2];
    } else {
        n = std::sqrt(n);
        const float a = (float)std::sqrt(r.rel_dim.x / r.rel_dim.y);
        bpd[0] = (int32_t)std::ceil(n * a);
        bpd[1] = (int32_t)std::ceil(n / a);
        count = bpd[0] * bpd[1];
    }
    for (int a = 0; a < 3; a++) {
        c.lbb[a] = 0.0;
        c.tfr[a] = (a < c.dimensionality ? (double)d * (double)bpd[a] : 0.0) + c.lbb[a];
    }
    c.time_step = 0.0001;  // HostData.timeStep
    c.capacity = count;
    c.use_gas_exchange = 0;
    c.use_flow = 0;
    c.increment_path = 0;
    c.precision = CB_PRECISION_FP64;
    c.use_graph = 1;
    if (in.has("gb300")) {
        const cbj::Value &g = in["gb300"];
        if (g.has("precision")) c.precision = precision_code(g["precision"].string());
        if (g.has("graph")) c.use_graph = g["graph"].integer() != 0;
        // linear shear along x over the last axis instead of the flow box, in
        // the units of flow.velocity (scaled by f0/mu0 like it); applies when
        // flow.impose is 1
        if (g.has("shear")) c.shear_speed = g["shear"].number() * c.f0_per_mu0;
    }
    if (precision_override >= 0) c.precision = precision_override;
    if (graph_override >= 0) c.use_graph = graph_override;
    check(cb_create(&c, &r.ctx), "cb_create");
    std::printf("==============\nInitialization\n==============\n");
    print_device();
    std::printf("bubbles %d (%d x %d x %d), box (%g, %g, %g), %s form\n", count, bpd[0], bpd[1],
                c.dimensionality == 3 ? bpd[2] : 1, c.tfr[0], c.tfr[1], c.tfr[2],
                precision_name(c.precision));

    // starting data: the reference's cuRAND MTGP32 draws in its order
    // (src/simulator.cu:676-692); the normal draw needs an even length
    const size_t cnt = (size_t)count, cnt2 = cnt + (cnt & 1);
    double *dev = nullptr;
    check_cuda(cudaMalloc(&dev, 5 * cnt2 * sizeof(double)), "cudaMalloc");
    double *dz = dev, *dx = dev + cnt2, *dy = dev + 2 * cnt2, *dw = dev + 3 * cnt2,
           *dr = dev + 4 * cnt2;
    curandGenerator_t gen;
    check_curand(curandCreateGenerator(&gen, CURAND_RNG_PSEUDO_MTGP32), "curandCreateGenerator");
    check_curand(curandSetPseudoRandomGeneratorSeed(gen, (unsigned long long)in["rngSeed"]["value"].number()),
                 "curandSetPseudoRandomGeneratorSeed");
    if (c.dimensionality == 3) check_curand(curandGenerateUniformDouble(gen, dz, cnt), "uniform z");
    check_curand(curandGenerateUniformDouble(gen, dx, cnt), "uniform x");
    check_curand(curandGenerateUniformDouble(gen, dy, cnt), "uniform y");
    check_curand(curandGenerateUniformDouble(gen, dw, cnt), "uniform w");
    check_curand(curandGenerateNormalDouble(gen, dr, cnt2, r.avg_rad,
                                            bubbles["radius"]["std"].number()),
                 "normal r");
    check_curand(curandDestroyGenerator(gen), "curandDestroyGenerator");
    std::vector<double> hz(cnt, 0.0), hx(cnt), hy(cnt), hw(cnt), hr(cnt);
    if (c.dimensionality == 3)
        check_cuda(cudaMemcpy(hz.data(), dz, cnt * 8, cudaMemcpyDeviceToHost), "copy z");
    check_cuda(cudaMemcpy(hx.data(), dx, cnt * 8, cudaMemcpyDeviceToHost), "copy x");
    check_cuda(cudaMemcpy(hy.data(), dy, cnt * 8, cudaMemcpyDeviceToHost), "copy y");
    check_cuda(cudaMemcpy(hw.data(), dw, cnt * 8, cudaMemcpyDeviceToHost), "copy w");
    check_cuda(cudaMemcpy(hr.data(), dr, cnt * 8, cudaMemcpyDeviceToHost), "copy r");
    cudaFree(dev);
    double ain = 0.0, max_r = 0.0;
    check(cb_assign_lattice(r.ctx, bpd, r.avg_rad, hx.data(), hy.data(), hz.data(), hw.data(),
                            hr.data(), count, &ain, &max_r),
          "cb_assign_lattice");
    check(cb_set_average_area(r.ctx, ain), "cb_set_average_area");
    r.cfg.average_surface_area_in = ain;

    std::printf("First neighbor search\n");
    check(cb_search_neighbors(r.ctx), "cb_search_neighbors");
    std::printf("Calculating initial velocities for Adams-Bashforth-Moulton\n");
    check(cb_bootstrap(r.ctx), "cb_bootstrap");
    std::printf("Stabilizing a few rounds after creation\n");
    for (int i = 0; i < 5; i++) stabilize(r, r.stabilization_steps);

    // box rescale to the target gas fraction (src/simulator.cu:793-833)
    std::printf("Scaling the simulation box\n");
    double bubble_volume = 0.0;
    check(cb_total_volume(r.ctx, &bubble_volume), "cb_total_volume");
    std::printf("Current phi: %.9g, target phi: %.9g\n", bubble_volume / box_volume(r.cfg), r.phi);
    check(cb_transform_positions(r.ctx, 1), "cb_transform_positions");
    Vec3 rel = r.rel_dim;
    double t = bubble_volume / (r.phi * rel.x * rel.y);
    if (c.dimensionality == 3) {
        t /= rel.z;
        t = std::cbrt(t);
    } else {
        t = std::sqrt(t);
        rel.z = 0.0;
    }
    const double rv[3] = {rel.x, rel.y, rel.z};
    double lbb[3], tfr[3], flow_lbb[3], flow_tfr[3];
    for (int a = 0; a < 3; a++) {
        lbb[a] = r.cfg.lbb[a];
        tfr[a] = t * rv[a];
        const double iv = tfr[a] - lbb[a];
        flow_tfr[a] = iv * r.cfg.flow_tfr[a] + lbb[a];
        flow_lbb[a] = iv * r.cfg.flow_lbb[a] + lbb[a];
    }
    for (int a = 0; a < 3; a++) {
        r.cfg.tfr[a] = tfr[a];
        r.cfg.flow_lbb[a] = flow_lbb[a];
        r.cfg.flow_tfr[a] = flow_tfr[a];
    }
    double mult = r.phi * box_volume(r.cfg) / kPi;
    mult = c.dimensionality == 3 ? std::cbrt(0.75 * mult) : std::sqrt(mult);
    r.cfg.bubble_volume_multiplier = mult;
    check(cb_set_box(r.ctx, lbb, tfr, mult, flow_lbb, flow_tfr), "cb_set_box");
    check(cb_transform_positions(r.ctx, 0), "cb_transform_positions");
    std::printf("Current phi: %.9g, target phi: %.9g\n", bubble_volume / box_volume(r.cfg), r.phi);
    std::printf("Neighbor search after scaling\n");
    check(cb_search_neighbors(r.ctx), "cb_search_neighbors");
    std::printf("Stabilizing a few rounds after scaling\n");
    for (int i = 0; i < 5; i++) stabilize(r, r.stabilization_steps);

    // energy-converged stabilisation (src/simulator.cu:858-902)
    std::printf("\n=============\nStabilization\n=============\n");
    std::printf("%-7s %-11s %-11s %-11s %-9s\n", "#steps", "dE", "e1", "e2", "#searches");
    int32_t num_steps = 0;
    const int32_t failsafe = 500;
    int64_t searches0 = report(r).searches;
    for (;;) {
        set_time(r, 0, 0.0);
        stabilize(r, r.stabilization_steps);
        const cb_report rep = report(r);
        const double time = ((double)rep.time_integer + rep.time_fraction) * r.time_scaling;
        double de = std::abs(r.energy2 - r.energy1);
        if (de > 0.0) de *= 2.0 / ((r.energy2 + r.energy1) * time);
        const bool stop = de < r.max_delta_energy || (r.energy2 < 1.0 && de < 0.1);
        if (stop) {
            std::printf("Final energies:\nbefore: %9.5e\nafter: %9.5e\ndelta: %9.5e\ntime: %9.5g\n",
                        r.energy1, r.energy2, de, time);
            break;
        } else if (num_steps > failsafe) {
            std::printf("Over %d steps taken and required delta energy not reached. "
                        "Constraints might be too strict.\n",
                        num_steps);
            break;
        }
        std::printf("%-7d %-9.5e %-9.5e %-9.5e %-9ld\n", (num_steps + 1) * r.stabilization_steps,
                    de, r.energy1, r.energy2, (long)(rep.searches - searches0));
        searches0 = rep.searches;
        ++num_steps;
    }
    check(cb_reset_rows(r.ctx, CB_RESET_WRAP | CB_RESET_ERROR), "cb_reset_rows");
    r.energy1 = energy(r);
    set_time(r, 0, 0.0);
    r.times_printed = 1;
}

// ------------------------------------------------------------- snapshots
// saveSnapshot, src/simulator.cu:387-512: per-bubble energies and a copy of
// the state now, the CSV written by an IO thread while the steps go on.
struct SnapData {
    int32_t count = 0;
    std::vector<double> x, y, z, r, vx, vy, vz, vr, path, error, energy;
    std::vector<int32_t> index;
    Vec3 interval;
};

void fetch_state(Run &r, SnapData &s) {
    cb_report rep = report(r);
    const size_t n = (size_t)rep.count;
    for (auto *v : {&s.x, &s.y, &s.z, &s.r, &s.vx, &s.vy, &s.vz, &s.vr, &s.path, &s.error, &s.energy})
        v->assign(n, 0.0);
    s.index.assign(n, 0);
    cb_state_view v;
    std::memset(&v, 0, sizeof(v));
    v.x = s.x.data(), v.y = s.y.data(), v.z = s.z.data(), v.r = s.r.data();
    v.dxdt = s.vx.data(), v.dydt = s.vy.data(), v.dzdt = s.vz.data(), v.drdt = s.vr.data();
    v.path = s.path.data(), v.error = s.error.data(), v.index = s.index.data();
    check(cb_get_state(r.ctx, &v), "cb_get_state");
    check(cb_bubble_energies(r.ctx, s.energy.data(), (int32_t)n), "cb_bubble_energies");
    s.count = v.count;
    s.interval.x = r.cfg.tfr[0] - r.cfg.lbb[0];
    s.interval.y = r.cfg.tfr[1] - r.cfg.lbb[1];
    s.interval.z = r.cfg.tfr[2] - r.cfg.lbb[2];
}

void write_snapshot(const SnapData &s, const std::string &name, uint32_t num,
                    std::vector<double> *px, std::vector<double> *py, std::vector<double> *pz) {
    std::stringstream ss;
    ss << name << ".csv." << num;
    std::ofstream file(ss.str().c_str(), std::ios::out);
    if (!file.is_open()) return;
    file.precision(g_output_digits);
    file << "x,y,z,r,vx,vy,vz,vtot,vr,path,energy,displacement,error,index\n";
    for (int32_t i = 0; i < s.count; ++i) {
        const int32_t ind = s.index[i];
        const double xi = s.x[i], yi = s.y[i], zi = s.z[i];
        const double vxi = s.vx[i], vyi = s.vy[i], vzi = s.vz[i];
        // displacement since the previous snapshot, as the reference writes it
        double dX = std::abs(xi - (*px)[ind]);
        dX = dX > 0.5 * s.interval.x ? dX - s.interval.x : dX;
        double dY = std::abs(yi - (*py)[ind]);
        dY = dY > 0.5 * s.interval.y ? dY - s.interval.y : dY;
        double dZ = std::abs(zi - (*pz)[ind]);
        dZ = dZ > 0.5 * s.interval.z ? dZ - s.interval.z : dZ;
        file << xi - 0.5 * s.interval.x << "," << yi - 0.5 * s.interval.y << ","
             << zi - 0.5 * s.interval.z << "," << s.r[i] << "," << vxi << "," << vyi << ","
             << vzi << "," << std::sqrt(vxi * vxi + vyi * vyi + vzi * vzi) << "," << s.vr[i]
             << "," << s.path[i] << "," << s.energy[i] << ","
             << std::sqrt(dX * dX + dY * dY + dZ * dZ) << "," << s.error[i] << "," << ind
             << "\n";
        (*px)[ind] = xi;
        (*py)[ind] = yi;
        (*pz)[ind] = zi;
    }
}

void save_snapshot(Run &r) {
    if (r.io.joinable()) r.io.join();
    auto data = std::make_shared<SnapData>();
    fetch_state(r, *data);
    const uint32_t num = r.num_snapshots++;
    r.io = std::thread([data, num, &r]() {
        write_snapshot(*data, r.snapshot_name, num, &r.prev_x, &r.prev_y, &r.prev_z);
    });
}

// Starting positions by bubble index (src/simulator.cu:904-937).
void init_previous(Run &r) {
    SnapData s;
    fetch_state(r, s);
    const size_t cap = (size_t)r.cfg.capacity;
    r.prev_x.assign(cap, 0.0);
    r.prev_y.assign(cap, 0.0);
    r.prev_z.assign(cap, 0.0);
    for (int32_t i = 0; i < s.count; i++) {
        r.prev_x[s.index[i]] = s.x[i];
        r.prev_y[s.index[i]] = s.y[i];
        r.prev_z[s.index[i]] = s.z[i];
    }
}

// ------------------------------------------------------------ checkpoint
// The complete AB2 state, the pair list, the clock and the simulation
// loop's host data, so that a resumed run continues step for step. Not in
// the reference.
constexpr char kMagic[8] = {'C', 'B', 'G', 'C', 'K', 'P', 'T', '1'};

template <typename T>
void put(std::ofstream &f, const T &v) {
    f.write(reinterpret_cast<const char *>(&v), sizeof(T));
}
template <typename T>
void put_vec(std::ofstream &f, const std::vector<T> &v) {
    put(f, (uint64_t)v.size());
    f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}
template <typename T>
void get(std::ifstream &f, T &v) {
    f.read(reinterpret_cast<char *>(&v), sizeof(T));
    if (!f) throw std::runtime_error("checkpoint truncated");
}
template <typename T>
void get_vec(std::ifstream &f, std::vector<T> &v) {
    uint64_t n = 0;
    get(f, n);
    v.resize(n);
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(T)));
    if (!f) throw std::runtime_error("checkpoint truncated");
}

struct FullState {
    std::vector<double> d[18];
    std::vector<int32_t> i[5];
};

cb_state_view view_of(FullState &s, int32_t count) {
    cb_state_view v;
    std::memset(&v, 0, sizeof(v));
    v.count = count;
    double **dp[18] = {&v.x, &v.y, &v.z, &v.r, &v.dxdt, &v.dydt, &v.dzdt, &v.drdt, &v.dxdto,
                       &v.dydto, &v.dzdto, &v.drdto, &v.path, &v.error, &v.saved_x, &v.saved_y,
                       &v.saved_z, &v.saved_r};
    int32_t **ip[5] = {&v.wrap_count_x, &v.wrap_count_y, &v.wrap_count_z, &v.index,
                       &v.num_neighbors};
    for (int q = 0; q < 18; q++) *dp[q] = s.d[q].data();
    for (int q = 0; q < 5; q++) *ip[q] = s.i[q].data();
    return v;
}

void write_checkpoint(Run &r, const std::string &path) {
    const cb_report rep = report(r);
    FullState s;
    for (auto &v : s.d) v.assign((size_t)std::max(rep.count, 1), 0.0);
    for (auto &v : s.i) v.assign((size_t)std::max(rep.count, 1), 0);
    cb_state_view v = view_of(s, rep.count);
    check(cb_get_state(r.ctx, &v), "cb_get_state");
    std::vector<int32_t> pi((size_t)std::max(rep.num_pairs, 1)), pj(pi.size());
    int32_t np = 0;
    check(cb_get_pairs(r.ctx, pi.data(), pj.data(), (int32_t)pi.size(), &np), "cb_get_pairs");
    pi.resize((size_t)np);
    pj.resize((size_t)np);
    const std::string tmp = path + ".tmp";
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f) throw std::runtime_error("cannot write " + tmp);
        f.write(kMagic, 8);
        put(f, r.cfg);
        put(f, rep);
        put(f, r.avg_rad), put(f, r.phi), put(f, r.time_scaling), put(f, r.energy1);
        put(f, r.energy2), put(f, r.snapshot_frequency), put(f, r.min_num_bubbles);
        put(f, r.times_printed), put(f, r.num_snapshots), put(f, (int32_t)r.add_flow);
        put(f, r.rel_dim);
        put_vec(f, std::vector<char>(r.snapshot_name.begin(), r.snapshot_name.end()));
        for (auto &q : s.d) {
            q.resize((size_t)rep.count);
            put_vec(f, q);
        }
        for (auto &q : s.i) {
            q.resize((size_t)rep.count);
            put_vec(f, q);
        }
        put_vec(f, pi);
        put_vec(f, pj);
        put_vec(f, r.prev_x), put_vec(f, r.prev_y), put_vec(f, r.prev_z);
    }
    std::rename(tmp.c_str(), path.c_str());
}

void read_checkpoint(Run &r, const std::string &path, int graph_override) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot read " + path);
    char magic[8];
    f.read(magic, 8);
    if (!f || std::memcmp(magic, kMagic, 8) != 0) throw std::runtime_error("not a checkpoint");
    cb_report rep{};
    int32_t add_flow = 0;
    get(f, r.cfg);
    get(f, rep);
    get(f, r.avg_rad), get(f, r.phi), get(f, r.time_scaling), get(f, r.energy1);
    get(f, r.energy2), get(f, r.snapshot_frequency), get(f, r.min_num_bubbles);
    get(f, r.times_printed), get(f, r.num_snapshots), get(f, add_flow);
    get(f, r.rel_dim);
    std::vector<char> name;
    get_vec(f, name);
    r.snapshot_name.assign(name.begin(), name.end());
    r.add_flow = add_flow != 0;
    FullState s;
    for (auto &q : s.d) get_vec(f, q);
    for (auto &q : s.i) get_vec(f, q);
    std::vector<int32_t> pi, pj;
    get_vec(f, pi);
    get_vec(f, pj);
    get_vec(f, r.prev_x), get_vec(f, r.prev_y), get_vec(f, r.prev_z);
    if (graph_override >= 0) r.cfg.use_graph = graph_override;
    check(cb_create(&r.cfg, &r.ctx), "cb_create");
    cb_state_view v = view_of(s, rep.count);
    check(cb_load_state(r.ctx, &v), "cb_load_state");
    check(cb_set_pairs(r.ctx, pi.data(), pj.data(), (int32_t)pi.size()), "cb_set_pairs");
    check(cb_set_time(r.ctx, rep.time_step, rep.time_integer, rep.time_fraction), "cb_set_time");
}

// ------------------------------------------------------------- simulate()
bool time_reached(const cb_report &rep, uint64_t ti, double tf) {
    return rep.time_integer > ti || (rep.time_integer == ti && rep.time_fraction >= tf);
}

void split_time(double t, uint64_t &ti, double &tf) {
    ti = (uint64_t)t;
    tf = t - (double)ti;
}

void simulate(Run &r) {
    if (r.snapshot_frequency > 0.0) {
        if (r.prev_x.empty()) init_previous(r);
        if (r.num_snapshots == 0) save_snapshot(r);
    }
    std::printf("\n===========\nIntegration\n===========\n");
    std::printf("%-5s %-8s %-6s %-11s %9s %10s %-6s %-9s %-11s %-11s %-11s \n", "T", "phi", "R",
                "dE", "#b   ", "#pairs", "#steps", "#searches", "min ts", "max ts", "avg ts");
    check(cb_set_options(r.ctx, 1, r.add_flow ? 1 : 0, 1), "cb_set_options");
    check(cb_reset_rows(r.ctx, CB_RESET_DT_STATS), "cb_reset_rows");
    const double ix = r.cfg.tfr[0] - r.cfg.lbb[0], iy = r.cfg.tfr[1] - r.cfg.lbb[1],
                 iz = r.cfg.tfr[2] - r.cfg.lbb[2];
    const double min_interval = r.cfg.dimensionality == 3 ? 0.5 * std::min(ix, std::min(iy, iz))
                                                          : 0.5 * std::min(ix, iy);
    bool cont = true;
    int64_t steps_in_time_step = 0, total = 0;
    cb_report rep = report(r);
    int64_t searches0 = rep.searches;
    // CUBBLE_PROFILE: start here; stop after 1000 steps in a time unit or
    // once the loop has printed (the reference's timesPrinted == 2)
    bool profiling = false;
    if (g_profile_range) profiling = cudaProfilerStart() == cudaSuccess;
    constexpr int64_t kProfileSteps = 1000;
    while (cont) {
        // the next output time: a printed time unit or a snapshot
        uint64_t pi = 0, si = 0;
        double pf = 0.0, sf = 0.0;
        split_time(r.times_printed / r.time_scaling, pi, pf);
        cb_stop stop;
        std::memset(&stop, 0, sizeof(stop));
        stop.time_integer = pi;
        stop.time_fraction = pf;
        const bool snaps = r.snapshot_frequency > 0.0;
        if (snaps) {
            split_time(r.num_snapshots / (r.snapshot_frequency * r.time_scaling), si, sf);
            if (si < pi || (si == pi && sf < pf)) {
                stop.time_integer = si;
                stop.time_fraction = sf;
            }
        }
        stop.min_count = r.min_num_bubbles;
        stop.max_radius = min_interval;
        int64_t limit = r.max_steps > 0 ? r.max_steps - total : INT64_MAX / 2;
        if (profiling) limit = std::min(limit, kProfileSteps - steps_in_time_step);
        const int64_t steps0 = rep.steps;
        check(cb_integrate_until(r.ctx, limit, &stop, &rep), "cb_integrate_until");
        const int64_t k = rep.steps - steps0;
        total += k;
        cont = rep.count > r.min_num_bubbles && rep.max_radius < min_interval;
        bool reset_errors = false;
        if (time_reached(rep, pi, pf)) {
            // steps counted up to, not including, this printing step
            const int64_t shown = steps_in_time_step + k - 1;
            r.energy2 = energy(r);
            double de = std::abs(r.energy2 - r.energy1);
            if (de > 0.0) de *= 2.0 / (r.energy2 + r.energy1);
            double avg[6];
            check(cb_averages(r.ctx, avg), "cb_averages");
            const double rel_rad = avg[0] / r.avg_rad;
            std::ofstream res("results.dat", std::ios_base::app);
            res.precision(g_output_digits);
            if (res.is_open()) {
                const double vx = avg[1], vy = avg[2], vz = avg[3], vr = avg[4];
                res << r.times_printed << " " << rel_rad << " " << rep.count << " " << avg[5] << " "
                    << r.energy2 << " " << de << " " << vx << " " << vy << " " << vz << " "
                    << std::sqrt(vx * vx + vy * vy + vz * vz) << " " << vr << "\n";
            } else {
                std::printf("Couldn't open file stream to append results to!\n");
            }
            double vol = 0.0;
            check(cb_total_volume(r.ctx, &vol), "cb_total_volume");
            const double phi = vol / box_volume(r.cfg);
            std::printf("%-5d ", r.times_printed);
            std::printf("%-#8.6g ", phi);
            std::printf("%-#6.4g ", rel_rad);
            std::printf("%-9.5e ", de);
            std::printf("%9d ", rep.count);
            std::printf("%10d ", rep.num_pairs);
            std::printf("%6ld ", (long)shown);
            std::printf("%-9ld ", (long)(rep.searches - searches0));
            std::printf("%-9.5e ", rep.dt_min);
            std::printf("%-9.5e ", rep.dt_max);
            std::printf("%-9.5e \n", shown > 0 ? rep.dt_sum / shown : rep.dt_sum);
            std::fflush(stdout);
            ++r.times_printed;
            steps_in_time_step = 1;
            r.energy1 = r.energy2;
            searches0 = rep.searches;
            check(cb_reset_rows(r.ctx, CB_RESET_DT_STATS), "cb_reset_rows");
            reset_errors = true;
        } else {
            steps_in_time_step += k;
        }
        if (snaps && time_reached(rep, si, sf)) save_snapshot(r);
        if (reset_errors) {
            check(cb_reset_rows(r.ctx, CB_RESET_ERROR), "cb_reset_rows");
            if (!r.checkpoint.empty()) write_checkpoint(r, r.checkpoint);
        }
        if (profiling && (steps_in_time_step >= kProfileSteps || r.times_printed >= 2)) {
            cudaProfilerStop();
            profiling = false;
        }
        if (r.max_steps > 0 && total >= r.max_steps) break;
    }
    if (profiling) cudaProfilerStop();
    if (rep.count <= r.min_num_bubbles) {
        std::printf("Stopping simulation, since the number of bubbles left in the simulation (%d) "
                    "is less than or equal to the specified minimum (%d)\n",
                    rep.count, r.min_num_bubbles);
    } else if (rep.max_radius > min_interval) {
        std::printf("Stopping simulation, since the radius of the largest bubble (%g) is greater "
                    "than the simulation box (%g, %g, %g)\n",
                    rep.max_radius, ix, iy, iz);
    } else if (r.max_steps > 0 && total >= r.max_steps) {
        std::printf("Stopping simulation after %ld integration steps (--max-steps)\n", (long)total);
    } else {
        std::printf("Stopping simulation for an unknown reason...\n");
    }
    if (r.snapshot_frequency > 0.0) save_snapshot(r);
    if (r.io.joinable()) r.io.join();
}

// ------------------------------------------------------------ array jobs
// array.params: every {...} block is one job; each line "a.b.c = value"
// overrides the input's value at that path, keeping its type
// (scripts/triton/array_job.py:54-75, :147-158).
std::vector<cbj::Value> expand_array(const cbj::Value &base, const std::string &text) {
    std::vector<cbj::Value> jobs;
    size_t p = 0;
    for (;;) {
        const size_t a = text.find('{', p);
        if (a == std::string::npos) break;
        const size_t b = text.find('}', a);
        if (b == std::string::npos) throw std::runtime_error("array file: unterminated '{'");
        cbj::Value job = base;
        std::istringstream lines(text.substr(a + 1, b - a - 1));
        std::string line;
        while (std::getline(lines, line)) {
            const size_t eq = line.find('=');
            if (eq == std::string::npos) continue;
            auto trim = [](std::string s) {
                const size_t i = s.find_first_not_of(" \t\r");
                const size_t j = s.find_last_not_of(" \t\r");
                return i == std::string::npos ? std::string() : s.substr(i, j - i + 1);
            };
            const std::string key = trim(line.substr(0, eq)), value = trim(line.substr(eq + 1));
            if (key.empty()) continue;
            std::vector<std::string> path;
            std::stringstream ks(key);
            std::string part;
            while (std::getline(ks, part, '.')) path.push_back(part);
            cbj::Value &dst = job.at_path(path);
            if (dst.kind == cbj::Value::String) {
                dst.str = value;
            } else if (dst.kind == cbj::Value::Bool) {
                dst.b = value == "true" || value == "1";
            } else {
                dst.kind = cbj::Value::Number;
                dst.num = std::strtod(value.c_str(), nullptr);
            }
        }
        jobs.push_back(job);
        p = b + 1;
    }
    if (jobs.empty()) throw std::runtime_error("array file holds no '{' block");
    return jobs;
}

std::string read_file(const std::string &path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("Couldn't open input file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

int run_one(const cbj::Value &in, int precision, int graph, int64_t max_steps,
            const std::string &checkpoint, const std::string &resume) {
    Run r;
    r.max_steps = max_steps;
    r.checkpoint = checkpoint;
    if (!resume.empty()) {
        read_checkpoint(r, resume, graph);
        std::printf("Resumed from %s at printed time unit %u\n", resume.c_str(), r.times_printed);
    } else {
        init(r, in, precision, graph);
    }
    simulate(r);
    cb_destroy(r.ctx);
    std::printf("Done\n");
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    std::string input, array, checkpoint, resume;
    int precision = -1, graph = -1;
    int64_t max_steps = -1;
    for (int a = 1; a < argc; a++) {
        const std::string s = argv[a];
        auto next = [&]() -> std::string {
            if (a + 1 >= argc) throw std::runtime_error("missing value after " + s);
            return argv[++a];
        };
        try {
            if (s == "--precision") {
                const std::string v = next();
                precision = precision_code(v);
            } else if (s == "--no-graph") {
                graph = 0;
            } else if (s == "--checkpoint") {
                checkpoint = next();
            } else if (s == "--resume") {
                resume = next();
            } else if (s == "--max-steps") {
                max_steps = std::stoll(next());
            } else if (s == "--output-digits") {
                g_output_digits = std::stoi(next());
                if (g_output_digits < 1 || g_output_digits > 17)
                    throw std::runtime_error("--output-digits must be 1 ... 17");
            } else if (s == "--array") {
                array = next();
            } else if (s == "--profile-range") {
                g_profile_range = true;
            } else if (input.empty()) {
                input = s;
            } else {
                throw std::runtime_error("unexpected argument " + s);
            }
        } catch (const std::exception &e) {
            std::printf("%s\n", e.what());
            return EXIT_FAILURE;
        }
    }
    if (input.empty() && resume.empty()) {
        std::printf("Usage: %s inputFile\n\twhere inputFile is the name of the (.json) file "
                    "containing the simulation input.\n",
                    argv[0]);
        return EXIT_FAILURE;
    }
    int ngpu = 0;
    if (cudaGetDeviceCount(&ngpu) != cudaSuccess || ngpu < 1) {
        std::printf("No CUDA capable devices found.\n");
        return EXIT_FAILURE;
    }
    try {
        if (!array.empty()) {
            const cbj::Value base = cbj::parse(read_file(input));
            const std::vector<cbj::Value> jobs = expand_array(base, read_file(array));
            char cwd[4096];
            if (!getcwd(cwd, sizeof(cwd))) throw std::runtime_error("getcwd failed");
            for (size_t k = 0; k < jobs.size(); k++) {
                const std::string dir = std::string(cwd) + "/run_" + std::to_string(k);
                mkdir(dir.c_str(), 0755);
                if (chdir(dir.c_str()) != 0) throw std::runtime_error("cannot enter " + dir);
                std::printf("---- array job %zu of %zu in %s\n", k + 1, jobs.size(), dir.c_str());
                run_one(jobs[k], precision, graph, max_steps, checkpoint, std::string());
                if (chdir(cwd) != 0) throw std::runtime_error("cannot return to " + std::string(cwd));
            }
            return EXIT_SUCCESS;
        }
        const cbj::Value in = resume.empty() ? cbj::parse(read_file(input)) : cbj::Value();
        run_one(in, precision, graph, max_steps, checkpoint, resume);
    } catch (const std::exception &e) {
        std::printf("Error: %s\n", e.what());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
