// mflbm_main: the MF-LBM program on libmflbm.
//
// Runs in a case folder laid out as the reference's (input/job_status.txt,
// input/simulation_control.txt, input/Geometry_File_Path.txt, the geometry
// .dat) and writes the reference's results/ tree: the program of
// src/main.cpp:31-366 with its parameter reading (src/IO_multiphase.cpp:16-246,
// src/utils.cpp:17-153), geometry set-up (src/Misc.cpp:13-216), start-up
// (src/Init_multiphase.cpp:100-290, 501-537), monitors (src/Monitor.cpp:17-495)
// and output files, with every time step, reduction and output body computed
// on the GPU through the C ABI of mflbm.h.
//
//   mflbm_main [--fp64] [--strict] [case folder]
//
// The solver precision is the reference's compile-time choice
// (includes/solver_precision.h); here it is --fp64 (default FP32).  --strict
// selects the kernels whose arithmetic is the reference's IEEE sequence.
//
// Differences from the reference's program, by design:
//   * monitor sums are FP64 on the device (the reference sums serially in
//     the solver precision); the .dat files print them in the solver
//     precision with the reference's stream formatting;
//   * geometry_preprocess_cmd 1 (load precomputed boundary info) computes
//     it instead: the device preprocessing takes milliseconds;
//   * a geometry sample smaller than the domain is rejected (the reference
//     reads it with the domain's dimensions).
#include <sys/stat.h>
#include <unistd.h>

#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mflbm.h"

namespace {

[[noreturn]] void die(const std::string& msg) {
    std::cout << "Error: " << msg << std::endl;
    std::exit(1);
}

void check(int rc, const char* what) {
    if (rc != MFLBM_OK) die(std::string(what) + ": " + mflbm_last_error());
}

// ---- simulation_control.txt: first "name value" line whose name matches
struct Control {
    std::vector<std::pair<std::string, std::string>> kv;
    explicit Control(const std::string& path) {
        std::ifstream f(path);
        if (!f.good()) die("Missing simulation control file! Exiting program!");
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream s(line);
            std::string name, value;
            s >> name >> value;
            kv.emplace_back(name, value);
        }
    }
    const std::string& raw(const std::string& name) const {
        for (const auto& p : kv)
            if (p.first == name) return p.second;
        die("ERROR! Couldn't find the variable named: (" + name + ") in the file");
    }
    int i(const std::string& n) const { return std::stoi(raw(n)); }
    long long ll(const std::string& n) const { return std::stoll(raw(n)); }
};

template <class T> T parse_real(const std::string& s);
template <> float parse_real<float>(const std::string& s) { return std::stof(s); }
template <> double parse_real<double>(const std::string& s) { return std::stod(s); }

std::string read_string_key(const std::string& path, const std::string& name) {
    std::ifstream f(path);
    if (!f.good()) die("Error opening Geometry_File_Path.txt!");
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream s(line);
        std::string n, v;
        s >> n >> v;
        if (n == name) return v;
    }
    die("ERROR! Couldn't find the variable named: (" + name + ") in the file");
}

void mkdirs(const std::string& p) { mkdir(p.c_str(), 0755); }

// append (or create on the first monitor call) a results file and write one line
void put_line(const std::string& path, bool fresh, const std::string& line) {
    std::ofstream f(path, fresh ? std::ios_base::out : std::ios_base::app);
    if (!f.good()) die("Could not open " + path);
    f << line << std::endl;
}

template <class... A> std::string cat(const A&... a) {
    std::ostringstream s;
    int dummy[] = {0, ((s << a << ' '), 0)...};
    (void)dummy;
    std::string r = s.str();
    if (!r.empty()) r.pop_back();
    return r;
}

std::string vtk_name(const char* dir, const char* stem, int nt) {
    char b[256];
    snprintf(b, sizeof b, "results/out3.field_data/%s/%s%010d.vtk", dir, stem, nt);
    return b;
}

template <class T> struct Run {
    // ---- parameters (src/IO_multiphase.cpp:47-187)
    std::string job_status;
    int initial_fluid_distribution_option, breakthrough_check, steady_state_option, benchmark_cmd;
    int output_fieldData_precision_cmd, extreme_large_sim_cmd, modify_geometry_cmd, external_geometry_read_cmd;
    int geometry_dims_type_size, geometry_preprocess_cmd, porous_plate_cmd, change_inlet_fluid_phase_cmd;
    long long nx, ny, nz;
    int n_exclude_inlet, n_exclude_outlet, wall[6], iper, jper, kper;
    T la_nu1, la_nu2, lbm_gamma, theta, convergence_criteria, target_inject_pore_volume, ca_0, sa_inject;
    T interface_z0, force_z0, sa_target, checkpoint_save_timer, checkpoint_2rd_save_timer, simulation_duration_timer;
    T d_vol_animation, d_vol_detail, d_vol_monitor, RK_beta;
    int inlet_BC, outlet_BC, Z_porous_plate, ntime_max, ntime_visual, ntime_animation, ntime_monitor;
    int ntime_monitor_profile_ratio, ntime_monitor_profile, ntime_clock_sum, ntime_display_steps;
    int rho_in_new, rho_out_BC;
    // ---- state
    mflbm_control ctl{};
    mflbm_params prm{};
    mflbm_derived der{};
    mflbm_context* ctx = nullptr;
    std::vector<int> pore_profile_z;
    long long pore_sum = 0, pore_sum_effective = 0;
    int ntime0 = 1, ntime = 1, end_indicator = 0;
    T monitor_prev = T(0), monitor_cur = T(0);
    const T eps = std::numeric_limits<float>::epsilon();
    bool strict;

    explicit Run(bool strict_) : strict(strict_) {}

    void read_parameters() {
        std::ifstream js("input/job_status.txt");
        if (!js.good()) die("Missing job status file! Exiting program!");
        job_status.assign(std::istreambuf_iterator<char>(js), std::istreambuf_iterator<char>());
        if (job_status == "new_simulation") std::cout << "Simulation status is: New Simulation!" << std::endl;
        else if (job_status == "continue_simulation") std::cout << "Simulation status is: Continue existing simulation!" << std::endl;
        else die("Wrong simlation status! Exiting program!");
        const Control c("input/simulation_control.txt");
        auto R = [&](const char* n) { return parse_real<T>(c.raw(n)); };
        initial_fluid_distribution_option = c.i("initial_fluid_distribution_option");
        breakthrough_check = c.i("breakthrough_check");
        steady_state_option = c.i("steady_state_option");
        convergence_criteria = R("convergence_criteria");
        benchmark_cmd = c.i("benchmark_cmd");
        output_fieldData_precision_cmd = c.i("output_fieldData_precision_cmd");
        extreme_large_sim_cmd = c.i("extreme_large_sim_cmd");
        modify_geometry_cmd = c.i("modify_geometry_cmd");
        external_geometry_read_cmd = c.i("external_geometry_read_cmd");
        geometry_dims_type_size = c.i("geometry_dims_type_size");
        if (geometry_dims_type_size != 4 && geometry_dims_type_size != 8) die("Incorrect geometry_dims_type_size!");
        geometry_preprocess_cmd = c.i("geometry_preprocess_cmd");
        porous_plate_cmd = c.i("porous_plate_cmd");
        change_inlet_fluid_phase_cmd = c.i("change_inlet_fluid_phase_cmd");
        nx = c.ll("nxGlobal"); ny = c.ll("nyGlobal"); nz = c.ll("nzGlobal");
        n_exclude_inlet = c.i("n_exclude_inlet"); n_exclude_outlet = c.i("n_exclude_outlet");
        const char* wn[6] = {"domain_wall_status_x_min", "domain_wall_status_x_max", "domain_wall_status_y_min",
                             "domain_wall_status_y_max", "domain_wall_status_z_min", "domain_wall_status_z_max"};
        for (int k = 0; k < 6; ++k) wall[k] = c.i(wn[k]);
        iper = c.i("iper"); jper = c.i("jper"); kper = c.i("kper");
        la_nu1 = R("fluid1_viscosity"); la_nu2 = R("fluid2_viscosity");
        lbm_gamma = R("surface_tension"); theta = R("theta"); RK_beta = R("RK_beta");
        inlet_BC = c.i("inlet_BC"); outlet_BC = c.i("outlet_BC");
        target_inject_pore_volume = R("target_inject_pore_volume");
        ca_0 = R("capillary_number"); sa_inject = R("saturation_injection");
        interface_z0 = R("initial_interface_position"); force_z0 = R("body_force_0");
        sa_target = R("target_fluid1_saturation");
        Z_porous_plate = c.i("Z_porous_plate");
        ntime_max = c.i("max_time_step");
        (void)c.i("max_time_step_benchmark");
        ntime_visual = c.i("ntime_visual"); ntime_animation = c.i("ntime_animation");
        ntime_monitor = c.i("monitor_timer"); ntime_monitor_profile_ratio = c.i("monitor_profile_timer_ratio");
        ntime_clock_sum = c.i("computation_time_timer"); ntime_display_steps = c.i("display_steps_timer");
        checkpoint_save_timer = R("checkpoint_save_timer"); checkpoint_2rd_save_timer = R("checkpoint_2rd_save_timer");
        simulation_duration_timer = R("simulation_duration_timer");
        d_vol_animation = R("d_vol_animation"); d_vol_detail = R("d_vol_detail"); d_vol_monitor = R("d_vol_monitor");
        rho_in_new = c.i("rho_in_new"); rho_out_BC = c.i("rho_out_BC");
        (void)c.i("block_Threads_X"); (void)c.i("block_Threads_Y"); (void)c.i("block_Threads_Z");
        ntime_monitor_profile = ntime_monitor_profile_ratio * ntime_monitor;
        // checks of read_parameter_multi (src/IO_multiphase.cpp:200-242)
        int err = 0;
        if (theta > T(90)) {
            std::cout << "Error: contact angle is larger than 90 degrees! Please refer to the notes on 'simlation_control' file! Exiting program!" << std::endl;
            err = 1;
        }
        if (iper == 1 || wall[1] == 0 || wall[0] == 0) {
            std::cout << "Error: X direction periodic BC enabled or non-slip BC not applied at x = xmin or x = xmax! Exiting program!" << std::endl;
            err = 1;
        }
        if (jper == 0 && (wall[3] == 0 || wall[2] == 0)) {
            std::cout << "Error: non-slip BC not applied at y = ymin or y = ymax while y direction periodic BC not enabled! Exiting program!" << std::endl;
            err = 1;
        }
        if (jper == 1 && (wall[3] == 1 || wall[2] == 1)) {
            std::cout << "Error: non-slip BC applied at y = ymin or y = ymax while y direction periodic BC enabled! Exiting program!" << std::endl;
            err = 1;
        }
        if (kper == 1 && (wall[5] == 1 || wall[4] == 1)) {
            std::cout << "Error: non-slip BC applied at z = zmin or z = zmax while z direction periodic BC enabled! Exiting program!" << std::endl;
            err = 1;
        }
        if (outlet_BC == 1 && inlet_BC == 2) {
            std::cout << "Inlet/outlet boundary condition error: Inlet pressure + outlet convective BC is not supported! Exiting program!" << std::endl;
            err = 1;
        }
        if (err) die("Exit Program!");
        if (extreme_large_sim_cmd != 0) die("Extreme large simulation domain (extreme_large_sim_cmd = 1) is not supported yet!");
        // the hot path's keys
        ctl.nxGlobal = nx; ctl.nyGlobal = ny; ctl.nzGlobal = nz;
        ctl.iper = iper; ctl.jper = jper; ctl.kper = kper;
        ctl.domain_wall_status_x_min = wall[0]; ctl.domain_wall_status_x_max = wall[1];
        ctl.domain_wall_status_y_min = wall[2]; ctl.domain_wall_status_y_max = wall[3];
        ctl.domain_wall_status_z_min = wall[4]; ctl.domain_wall_status_z_max = wall[5];
        ctl.inlet_BC = inlet_BC; ctl.outlet_BC = outlet_BC;
        ctl.porous_plate_cmd = porous_plate_cmd; ctl.Z_porous_plate = Z_porous_plate;
        ctl.initial_fluid_distribution_option = initial_fluid_distribution_option;
        ctl.rho_out_BC = rho_out_BC;
        ctl.fluid1_viscosity = la_nu1; ctl.fluid2_viscosity = la_nu2;
        ctl.surface_tension = lbm_gamma; ctl.theta = theta; ctl.RK_beta = RK_beta;
        ctl.capillary_number = ca_0; ctl.saturation_injection = sa_inject;
        ctl.initial_interface_position = interface_z0; ctl.body_force_0 = force_z0;
    }

    // set_walls + read_walls + modify_geometry (src/Misc.cpp:13-186)
    std::vector<int32_t> walls_global() {
        std::vector<uint8_t> body;
        if (external_geometry_read_cmd == 1) {
            std::string path = read_string_key("input/Geometry_File_Path.txt", "geo_file_path_");
            while (!path.empty() && !isdigit((unsigned char)path.back())) path.pop_back();
            path += ".dat";
            FILE* f = fopen(path.c_str(), "rb");
            if (!f) die("Could not open the geometry file !");
            long long d[3] = {0, 0, 0};
            for (int k = 0; k < 3; ++k) {
                if (geometry_dims_type_size == 4) {
                    int v;
                    if (fread(&v, 4, 1, f) != 1) die("Could not load from the geometry file!");
                    d[k] = v;
                } else if (fread(&d[k], 8, 1, f) != 1) die("Could not load from the geometry file!");
            }
            std::cout << "Porous media sample size: nx = " << d[0] << ", ny = " << d[1] << ", nz = " << d[2] << std::endl;
            if (nx < d[0] || ny < d[1] || nz < d[2]) die("Error! Domain size is smaller than porous media sample size! Exiting program!");
            if (d[0] != nx || d[1] != ny || d[2] != nz)
                die("geometry sample smaller than the domain: the reference reads it with the domain's dimensions; pad the sample");
            body.resize((size_t)(nx * ny * nz));
            if (fread(body.data(), 1, body.size(), f) != body.size()) die("Could not load from the geometry file!");
            fclose(f);
        } else {
            std::cout << "This simulation does not use external geometry data!" << std::endl;
        }
        std::vector<int32_t> wg((size_t)(nx * ny * nz));
        check(mflbm_set_walls(&ctl, body.empty() ? nullptr : body.data(), wg.data()), "mflbm_set_walls");
        if (modify_geometry_cmd == 1) {
            const double xc = 0.5 * double(nx + 1), yc = 0.5 * double(ny + 1), zc = 0.5 * double(nz + 1);
            const double r1 = 0.25 * ny, r2 = ny * 0.5;
            const long long buffer = 10;
            for (long long k = 1; k <= nz; ++k)
                for (long long j = 1; j <= ny; ++j)
                    for (long long i = 1; i <= nx; ++i) {
                        const double d2 = pow(i - xc, 2) + pow(j - yc, 2) + pow(k - zc, 2);
                        const size_t s0 = (size_t)((i - 1) + nx * ((j - 1) + ny * (k - 1)));
                        if (d2 < pow(r1, 2)) wg[s0] = 1;
                        if (d2 > pow(r2, 2) && k > buffer && k < nz - buffer + 1) wg[s0] = 1;
                    }
            std::cout << "Internal geometry modified!" << std::endl;
        }
        return wg;
    }

    void setup() {
        const int prec = sizeof(T) == 4 ? MFLBM_FP32 : MFLBM_FP64;
        check(mflbm_params_from_control(&ctl, prec, strict ? MFLBM_STRICT : MFLBM_FAST, &prm, &der),
              "mflbm_params_from_control");
        for (const char* d : {"results", "results/out1.output", "results/out1.output/profile", "results/out2.checkpoint",
                              "results/out2.checkpoint/2rd_backup", "results/out3.field_data",
                              "results/out3.field_data/full_flow_field", "results/out3.field_data/phase_distribution"})
            mkdirs(d);
        std::vector<int32_t> wg = walls_global();
        check(mflbm_create(&prm, &ctx), "mflbm_create");
        std::vector<int32_t> walls((size_t)((nx + 4) * (ny + 4) * (nz + 4)));
        mflbm_geometry_counts counts{};
        check(mflbm_preprocess_geometry(ctx, wg.data(), walls.data(), nullptr, nullptr, nullptr, nullptr, &counts),
              "mflbm_preprocess_geometry");
        // pore profile (src/Misc.cpp:195-216) and info.txt (src/Init_multiphase.cpp:126-158)
        pore_profile_z.assign((size_t)nz, 0);
        auto s2 = [&](long long i, long long j, long long k) { return (size_t)((i + 1) + (nx + 4) * ((j + 1) + (ny + 4) * (k + 1))); };
        for (long long k = 1; k <= nz; ++k)
            for (long long j = 1; j <= ny; ++j)
                for (long long i = 1; i <= nx; ++i)
                    if (walls[s2(i, j, k)] <= 0) pore_profile_z[(size_t)(k - 1)]++;
        for (long long k = 1; k <= nz; ++k) pore_sum += pore_profile_z[(size_t)(k - 1)];
        for (long long k = 1 + n_exclude_inlet; k <= nz - n_exclude_outlet; ++k) pore_sum_effective += pore_profile_z[(size_t)(k - 1)];
        const T A_xy = T(der.A_xy);
        {
            std::ofstream fi("results/out1.output/info.txt");
            if (!fi.good()) die("Couldn't open the file results/out1.output/info.txt !");
            fi << " Grid information:" << std::endl;
            fi << "nxGlobal = " << nx << " , nyGlobal = " << ny << " , nzGlobal = " << nz << std::endl;
            fi << "Inlet open cross sectional area = " << A_xy << std::endl;
            fi << " Pore information:" << std::endl;
            fi << "Total number of pore nodes = " << pore_sum << std::endl;
            fi << "Total number of solid boundary nodes = " << counts.num_solid_boundary_global << std::endl;
            fi << "Total number of fluid boundary nodes = " << counts.num_fluid_boundary_global << std::endl;
            fi << "Total number of effective pore nodes (excluding inlet/outlet) = " << pore_sum_effective << std::endl;
            const T porosity_full = T(pore_sum) / T(((nx - 2) * (ny - 2) * (nz)));
            const T porosity_effective = T(pore_sum_effective) / ((nx - 2) * (ny - 2)) / T(nz - n_exclude_outlet - n_exclude_inlet);
            fi << "Full domain porosity = " << porosity_full << std::endl;
            fi << "Effective domain porosity  (excluding inlet/outlet) = " << porosity_effective << std::endl;
        }
        // timers from injected volumes (src/Init_multiphase.cpp:216-290)
        const bool open_v = inlet_BC == 1 && kper == 0 && wall[4] == 0 && wall[5] == 0;
        const T flowrate = T(der.flowrate);
        if (open_v && target_inject_pore_volume > T(0)) {
            ntime_max = int(T(target_inject_pore_volume * T(pore_sum)) / flowrate);
            if (ntime_max % 2 == 1) ntime_max = ntime_max + 1;
        }
        if (d_vol_animation > T(0) && open_v) {
            ntime_animation = int(T(d_vol_animation * T(pore_sum)) / flowrate);
            if (ntime_animation % 2 == 1) ntime_animation++;
        }
        if (d_vol_detail > T(0) && open_v) {
            ntime_visual = int(T(d_vol_detail * T(pore_sum)) / flowrate);
            if (ntime_visual % 2 == 1) ntime_visual++;
        }
        if (d_vol_monitor > T(0) && open_v) {
            ntime_monitor = int(T(d_vol_monitor * T(pore_sum)) / flowrate);
            if (ntime_monitor % 2 == 1) ntime_monitor++;
            ntime_monitor_profile = ntime_monitor_profile_ratio * ntime_monitor;
        }
        // fields
        std::vector<T> W_in((size_t)((nx + 2) * (ny + 2)));
        check(mflbm_inlet_profile(&ctl, prec, W_in.data()), "mflbm_inlet_profile");
        if (job_status == "new_simulation") {
            ntime0 = 1;
            check(mflbm_init_fields(ctx, initial_fluid_distribution_option, der.interface_z0, W_in.data()),
                  "mflbm_init_fields");
        } else {
            std::cout << "loading checkpoint data ... ";
            check(mflbm_read_checkpoint(ctx, "results/out2.checkpoint/id0000", W_in.data(), &ntime0),
                  "Checkpoint data not found or unreadable");
            check(mflbm_get_params(ctx, &prm), "mflbm_get_params");   // force_z, rho_in of the checkpoint
            std::cout << "Complete" << std::endl;
            // src/main.cpp:116-128: a new inlet (outlet) density for the pressure BC
            if (kper == 0 && wall[4] == 0 && wall[5] == 0 && inlet_BC == 2 && rho_in_new) {
                const T p_gradient = -force_z0 / T(3);
                mflbm_params p = prm;
                if (rho_out_BC) p.rho_out = (double)(T(1) - p_gradient * nz);
                else p.rho_in = (double)(T(p.rho_out) - p_gradient * nz);
                check(mflbm_set_params(ctx, &p), "mflbm_set_params");
                prm = p;
            }
        }
        if (change_inlet_fluid_phase_cmd != 0) change_inlet_fluid_phase();
        ntime = ntime0;
    }

    // src/Misc.cpp:277-384: move one component's populations onto the other for z <= interface_z0
    void change_inlet_fluid_phase() {
        const size_t n1 = (size_t)((nx + 2) * (ny + 2) * (nz + 2));
        std::vector<T> pdf(n1 * 38), phi((size_t)((nx + 8) * (ny + 8) * (nz + 8)));
        check(mflbm_download_fields(ctx, pdf.data(), phi.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                    nullptr, nullptr), "mflbm_download_fields");
        const int from = change_inlet_fluid_phase_cmd == 1 ? 1 : 0, to = 1 - from;
        for (long long k = 0; k <= nz + 1; ++k)
            for (long long j = 0; j <= ny + 1; ++j)
                for (long long i = 0; i <= nx - 1; ++i) {
                    if (!(k <= interface_z0)) continue;
                    const size_t s1 = (size_t)(i + (nx + 2) * (j + (ny + 2) * k));
                    for (int q = 0; q < 19; ++q) {
                        pdf[s1 + n1 * (q + 19 * to)] += pdf[s1 + n1 * (q + 19 * from)];
                        pdf[s1 + n1 * (q + 19 * from)] = T(0);
                    }
                }
        check(mflbm_upload_fields(ctx, pdf.data(), phi.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  nullptr, nullptr, nullptr), "mflbm_upload_fields");
        std::cout << "Inlet fluid phase was changed (1 to fluid1; 2 to fluid2): " << change_inlet_fluid_phase_cmd << std::endl;
    }

    bool first_monitor() const { return ntime0 == 1 && ntime == ntime_monitor; }

    // src/Monitor.cpp:17-272
    void monitor(const std::vector<double>& sl, const mflbm_monitor_ext& e) {
        auto S = [&](int m, long long k) { return sl[(size_t)m * nz + (size_t)k]; };  // k 0-based
        const bool fresh = first_monitor();
        const T ke1 = T(0.5) * T(e.usq1), ke2 = T(0.5) * T(e.usq2);
        const T umax_global = std::sqrt(T(e.umax2));
        double m1 = 0, m2 = 0, v1 = 0, v2 = 0;
        for (long long k = n_exclude_inlet; k < nz - n_exclude_outlet; ++k) {
            m1 += S(4, k); m2 += S(5, k); v1 += S(2, k); v2 += S(3, k);
        }
        const T saturation = T(v1 / (v1 + v2));
        put_line("results/out1.output/saturation.dat", fresh, cat(ntime, saturation, T(v1), T(v2), T(m1), T(m2)));
        double t1 = 0, t2 = 0, t3 = 0, t4 = 0;
        for (long long k = 0; k < nz; ++k) { t1 += S(4, k); t2 += S(5, k); t3 += S(2, k); t4 += S(3, k); }
        const T sat_full = T(t3 / (t3 + t4));
        double f1w = 0, f2w = 0, f1 = 0, f2 = 0;
        for (long long k = 0; k < nz; ++k) { f1w += S(0, k); f2w += S(1, k); }
        f1w /= double(nz); f2w /= double(nz);
        for (long long k = n_exclude_inlet; k < nz - n_exclude_outlet; ++k) { f1 += S(0, k); f2 += S(1, k); }
        f1 /= double(nz - n_exclude_outlet - n_exclude_inlet);
        f2 /= double(nz - n_exclude_outlet - n_exclude_inlet);
        const double fl_avg = f1 + f2;
        const T ca = T(fl_avg / der.A_xy) * la_nu1 / lbm_gamma;
        put_line("results/out1.output/Ca_number.dat", fresh, cat(ntime, ca, umax_global, ke1, ke2));
        put_line("results/out1.output/flowrate_time.dat", fresh,
                 cat(ntime, T(f1w + f2w), T(f1w), T(f2w), T(fl_avg), T(f1), T(f2)));
        put_line("results/out1.output/saturation_full_domain.dat", fresh, cat(ntime, sat_full, T(t3), T(t4), T(t1), T(t2)));
        if (kper == 0 && wall[4] == 0 && wall[5] == 0) {
            const T p1 = T(S(6, n_exclude_inlet)) / T(pore_profile_z[(size_t)n_exclude_inlet]);
            const T p2 = T(S(6, nz - n_exclude_outlet - 1)) / T(pore_profile_z[(size_t)(nz - n_exclude_outlet - 1)]);
            put_line("results/out1.output/pre.dat", fresh, cat(ntime, p1, p2, T(p1 - p2)));
        }
        if (ntime_monitor_profile > 0 && ntime % ntime_monitor_profile == 0) {
            char b[128];
            snprintf(b, sizeof b, "results/out1.output/profile/monitor %08d", ntime);
            std::ofstream f(b);
            for (long long k = 0; k < nz; ++k)
                f << T(k) << " " << T(S(0, k)) << " " << T(S(1, k)) << " " << T(S(4, k) / (S(4, k) + S(5, k))) << " "
                  << T(S(6, k) / (double(T(pore_profile_z[(size_t)k]) + eps))) << std::endl;
        }
        if (std::isnan(sat_full) || std::isnan(ca)) {
            std::cout << "Simulation failed due to NAN of saturation or capillary number" << std::endl;
            end_indicator = 3;
        } else if (umax_global > T(0.5)) {
            std::cout << "Simulation failed due to maximum velocity larger than 0.5 !" << std::endl;
            end_indicator = 3;
        }
        if (steady_state_option == 3) {
            monitor_prev = monitor_cur;
            monitor_cur = sat_full;
            const T err = std::fabs(monitor_cur - monitor_prev) / (std::fabs(monitor_cur) + eps);
            put_line("results/out1.output/steady_monitor_saturation_error.dat", fresh, cat(ntime, err));
            if (err < convergence_criteria && ntime > ntime_monitor) {
                std::cout << "Simulation converged based on saturation! Relative error = " << err
                          << " ; maximum velocity = " << umax_global << std::endl;
                end_indicator = 1;
            }
        }
        if (breakthrough_check == 1 && e.breakthrough >= 1) {
            end_indicator = 1;
            std::cout << "Breakthrough point reached! Exiting program!" << std::endl;
        }
    }

    // src/Monitor.cpp:277-351
    void monitor_phasefield(const mflbm_monitor_ext& e) {
        const T dphi = T(e.dphi_max);
        const T umax_global = std::sqrt(T(e.umax2));
        if (ntime > 0) {
            if (std::isnan(T(e.umax2)) || std::isnan(dphi)) {
                std::cout << "Simulation failed due to NAN!" << std::endl;
                end_indicator = 3;
                return;
            }
            put_line("results/out1.output/steady_monitor_max_phi_change.dat", first_monitor(), cat(ntime, dphi, umax_global));
            if (umax_global < 0.5) {
                if (dphi < convergence_criteria && ntime > ntime_monitor) {
                    std::cout << "Simulation converged based on maximum local change of phi! Relative error =    " << dphi
                              << "; maximum velocity =  " << umax_global << std::endl;
                    end_indicator = 1;
                }
            } else {
                std::cout << "Maximum velocity larger than 0.5, simulation failed!!!" << std::endl;
                end_indicator = 3;
            }
        }
    }

    // src/Monitor.cpp:355-441
    void monitor_capillary(const mflbm_monitor_ext& e) {
        const T umax_global = std::sqrt(T(e.umax2));
        const T pre_w = T(e.pre_w) / (T(e.n_w) + eps), pre_nw = T(e.pre_nw) / (T(e.n_nw) + eps);
        const T pc = (pre_nw - pre_w) / T(3);
        monitor_prev = monitor_cur;
        monitor_cur = pc;
        const T err = std::fabs(monitor_cur - monitor_prev) / (std::fabs(monitor_cur) + eps);
        put_line("results/out1.output/steady_monitor_capillary_pressure_error.dat", first_monitor(),
                 cat(ntime, err, pc, pre_w, pre_nw, err, umax_global));
        if (std::isnan(T(e.umax2)) || std::isnan(pc)) {
            std::cout << "Simulation failed due to NAN!" << std::endl;
            end_indicator = 3;
        } else if (umax_global < T(0.5)) {
            if (err < convergence_criteria && ntime > ntime_monitor) {
                std::cout << "Simulation converged based on change of capillary pressure! Relative error =   " << err
                          << " ; maximum velocity = " << umax_global << std::endl;
                end_indicator = 1;
            }
        } else {
            std::cout << "maximum velocity larger than 0.5, simulation failed!!!" << std::endl;
            end_indicator = 3;
        }
    }

    void save_checkpoint(int option) {
        check(mflbm_write_checkpoint(ctx, ntime, option == 0 ? "results/out2.checkpoint/id0000"
                                                             : "results/out2.checkpoint/2rd_backup/id0000"),
              "save_checkpoint");
        if (option == 0) {
            std::cout << "Saving checkpoint data completed!" << std::endl;
            put_line("./job_status.txt", true, "continue_simulation");
        } else {
            std::cout << "Saving secondary checkpoint data completed!" << std::endl;
        }
    }

    void vtk(int type) {
        const std::string p = type == 2 ? vtk_name("phase_distribution", "small_", ntime)
                                        : vtk_name("full_flow_field", "full_flow_field_", ntime);
        check(mflbm_write_vtk(ctx, type, output_fieldData_precision_cmd, p.c_str()), "VTK_legacy_writer_3D");
    }

    int main_loop() {
        if (job_status == "new_simulation" && benchmark_cmd == 0) {
            vtk(2);
            check(mflbm_write_walls_vtk(ctx, "results/out3.field_data/walls_bin.vtk"), "VTK_walls_bin");
        }
        const long long nodes = nx * ny * nz;
        std::vector<double> sl((size_t)(7 * nz));
        int counter_ck = 1, counter_ck2 = 1;
        auto clock = [] { return std::chrono::steady_clock::now(); };
        auto secs = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double>(b - a).count();
        };
        const auto t_loop = clock();
        auto t_sum = t_loop, t_disp = t_loop;
        const int last = ntime0 + ntime_max;
        auto next_multiple = [](int t, int m) { return m > 0 ? ((t + m - 1) / m) * m : 1 << 30; };
        auto hit = [](int t, int m) { return m > 0 && t % m == 0; };
        std::cout << "************************** Entering main loop *********************************" << std::endl;
        for (ntime = ntime0; ntime <= last;) {
            // run up to the next step with an output event as one graph-replayed stretch
            int ev = last;
            for (int m : {ntime_clock_sum, ntime_monitor, ntime_display_steps, ntime_animation, ntime_visual})
                ev = std::min(ev, next_multiple(ntime, m));
            check(mflbm_run(ctx, ntime, ev - ntime + 1), "main_iteration_kernel_GPU");
            ntime = ev;
            if (hit(ntime, ntime_clock_sum)) {
                check(mflbm_synchronize(ctx), "mflbm_synchronize");
                const auto t = clock();
                put_line("results/out1.output/time.dat", ntime0 == 1 && ntime == ntime_clock_sum,
                         cat(ntime, secs(t_sum, t), "sec"));
                t_sum = t;
            }
            if (hit(ntime, ntime_monitor)) {
                mflbm_monitor_ext e{};
                const bool track = steady_state_option == 2;
                check(mflbm_monitor_profile(ctx, sl.data(), &e, track ? 1 : 0), "monitor");
                if (steady_state_option == 0 || steady_state_option == 3) monitor(sl, e);
                else if (steady_state_option == 1) monitor_capillary(e);
                else if (steady_state_option == 2) monitor_phasefield(e);
            }
            if (hit(ntime, ntime_display_steps)) {
                check(mflbm_synchronize(ctx), "mflbm_synchronize");
                const auto t = clock();
                std::cout << "ntime =\t" << ntime << std::endl;
                std::cout << "simulation speed: " << double(nodes) * ntime_display_steps / (secs(t_disp, t) * 1e6) << " MLUPS" << std::endl;
                t_disp = t;
            }
            if (hit(ntime, ntime_animation)) vtk(2);
            if (hit(ntime, ntime_visual)) vtk(1);
            if (hit(ntime, ntime_clock_sum)) {
                const double hours = secs(t_loop, clock()) * 2.77777777777e-4;
                std::cout << "simulation has run\t" << hours << "\thours" << std::endl;
                if (hours >= simulation_duration_timer) {
                    std::cout << "Time to save checkpoint data and exit the program!" << std::endl;
                    end_indicator = 2;
                }
                bool ck = false, ck2 = false;
                if (hours >= counter_ck * checkpoint_save_timer) { ck = true; ++counter_ck; }
                if (hours >= counter_ck2 * checkpoint_2rd_save_timer) { ck2 = true; ++counter_ck2; }
                if (ck) save_checkpoint(0);
                if (ck2) save_checkpoint(1);
            }
            ++ntime;
            if (end_indicator > 0) { --ntime; break; }
        }
        check(mflbm_synchronize(ctx), "mflbm_synchronize");
        const double total = secs(t_loop, clock());
        std::cout << "************************** Exiting main iteration *********************************" << std::endl;
        std::cout << "Code speed:\t" << double(nodes) * double((ntime - ntime0) - 1) / (1e6 * total) << " MLUPS" << std::endl;
        if (end_indicator == 0) {
            ntime = ntime - 1;
            save_checkpoint(0);
            vtk(2);
            vtk(1);
            std::cout << "Simulation ended after\t" << ntime << " iterations which reached the maximum time step!" << std::endl;
            put_line("./job_status.txt", true, "simulation_reached_max_step");
        } else if (end_indicator == 1) {
            save_checkpoint(0);
            vtk(2);
            vtk(1);
            std::cout << "Simulation ended successfully after\t" << ntime << " iterations!" << std::endl;
            put_line("./job_status.txt", true, "simulation_done");
        } else if (end_indicator == 2) {
            save_checkpoint(0);
            std::cout << "Simulation data saved but not finished after\t" << ntime << " iterations!" << std::endl;
            put_line("./job_status.txt", true, "continue_simulation");
        } else {
            vtk(1);
            std::cout << "Simulation failed after\t" << ntime << " iterations!" << std::endl;
            put_line("./job_status.txt", true, "simulation_failed");
        }
        mflbm_destroy(ctx);
        std::cout << std::endl << "Code Finished " << std::endl;
        return 0;
    }
};

}  // namespace

int main(int argc, char** argv) {
    bool fp64 = false, strict = false;
    std::string dir;
    for (int a = 1; a < argc; ++a) {
        const std::string s = argv[a];
        if (s == "--fp64") fp64 = true;
        else if (s == "--strict") strict = true;
        else if (s == "--help" || s == "-h") {
            std::cout << "usage: mflbm_main [--fp64] [--strict] [case folder]" << std::endl;
            return 0;
        } else dir = s;
    }
    if (!dir.empty() && chdir(dir.c_str()) != 0) die("cannot enter " + dir);
    std::cout << "MF-LBM on libmflbm (GB300), " << (fp64 ? "FP64" : "FP32") << (strict ? ", strict arithmetic" : "") << std::endl;
    if (fp64) {
        Run<double> r(strict);
        r.read_parameters();
        r.setup();
        return r.main_loop();
    }
    Run<float> r(strict);
    r.read_parameters();
    r.setup();
    return r.main_loop();
}
