// gpat_run: replay driver for the engine.  Runs the per-frame sequence of
// solve_transport_equation (src/programs/stochastic-mhd.f90:312-567) through
// the C ABI only, with the reference's command-line switches for the options
// on the mover path (stochastic-mhd.f90:572-946).
//
//   gpat_run -dm data/ -cf conf.dat -ts 0 -te 20 -np 100000 -nm 1000000 ...
//
// Outputs in the diagnostics directory (-dd): quick.dat with the reference's
// columns (diagnostics.f90:116-170) and, per frame, fdists_XXXX.dat: int32
// npp, npp + 1 float64 bin edges, npp float64 weighted counts, npp uint64
// particle counts (the fglobal / pbins_edges_global datasets of
// fdists_XXXX.h5, without HDF5).  With -pd 1, particles_XXXX.dat per frame,
// and restart/particles_XXXX.dat at t_end always (dump_particles, see
// write_particles below).  With -tf .true. (particle tracking) the tags
// table is read from particle_tracking/<-ptf> under the diagnostics
// directory (int32 nrows, int32 nptl_tracking, the table in Fortran order)
// and particle_tracking/particles_tracked_XXXX.dat is written per frame
// (write_tracked below) instead of the distributions.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gpat_engine.h"

namespace {

struct Options {
    std::string dir_mhd_data = "data/", mhd_config_filename = "mhd_config.dat";
    std::string conf_file = "conf.dat", diagnostics_directory = "data/";
    long long nptl_max = 10000000, nptl = 10000;
    int time_interp_flag = 0, t_start = 0, t_end = 200, tmax_mhd = 100000;
    int single_time_frame = 0, dist_flag = 0, split_flag = 1, nsteps_interval = 10;
    int num_fine_steps = 1, ndim_field = 2, charge = -1, inject_new_ptl = 0;
    int inject_at_shock = 0, inject_part_box = 0, tmax_to_inject = 100000, check_drift_2d = 0;
    int particle_data_dump = 0;
    bool dump_escaped_dist = false, dump_escaped = false;   // -ded, -de (:939-946)
    // -tf, -ptf (stochastic-mhd.f90:711-722)
    bool track_particle_flag = false;
    std::string particle_tags_file = "tags_selected_01.dat";
    // -vdt, -rf, -qh, -ld, -sm (stochastic-mhd.f90:623-649, :839-842, :931-933)
    bool varying_dt_mhd = false, restart_flag = false, local_dist = false;
    double quota_hour = 48.0;
    int size_mpi_sub = 1;
    // inject_particles_at_large_* switches (stochastic-mhd.f90:735-806)
    bool inject_large_jz = false, inject_large_absj = false, inject_large_db2 = false;
    bool inject_large_divv = false, inject_large_rho = false, inject_same_nptl = false;
    double jz_min = 100.0, absj_min = 5.0, divv_min = 10.0, rho_min = 5.0, db2_min = 0.03;
    long long ncells_large_db2_norm = 800;
    int deltab_flag = 0, correlation_flag = 0;   // -db, -co (stochastic-mhd.f90:859-866)
    // -sc, -ug (stochastic-mhd.f90:883-890): Cartesian and non-uniform by
    // default, as the reference's CLI; -ug 1 for a uniform grid.
    int spherical_coord = 0, uniform_grid = 0;
    int include_3rd_dim = 0;   // -i3 (stochastic-mhd.f90:899-902)
    // acceleration surfaces (stochastic-mhd.f90:903-930)
    int acc_by_surface = 0;
    bool surface2_existed = false, is_intersection = true;
    std::string surface_filename1 = "sname_default", surface_filename2 = "sname_default";
    std::string surface_norm1 = "+y", surface_norm2 = "+y";
    long long ncells_large_jz_norm = 800, ncells_large_absj_norm = 800;
    long long ncells_large_divv_norm = 800, ncells_large_rho_norm = 800;
    double tinterval = 1e-7, power_index = 7.0, split_ratio = 2.72, pmin_split = 2.0;
    double particle_v0 = 5.0, drift_param1 = 4e7, drift_param2 = 2e8;
    // particle_mover's switches with the reference CLI's defaults
    // (stochastic-mhd.f90:631-641, :935-937): NLGC on, fixed kperp/kpara off.
    bool focused_transport = false, nlgc = true;
    double kperp_kpara = 0.01, duu_init = 10.0;
    // set_dpp_params switches (stochastic-mhd.f90:843-858)
    int dpp_wave = 0, dpp_shear = 0, weak_scattering = 0;
    double tau0_scattering = 1.0;
    double ptl_box[6] = {0.0, 0.0, 0.0, 1.0, 1.0, 1.0};   // xmin ymin zmin xmax ymax zmax
    // engine options
    int precision = GPAT_PREC_MIXED, noise = GPAT_NOISE_UNIFORM, device = 0, bin_interval = 0;
    bool precision_set = false;
    unsigned long long seed = 0x5EED0001ull;
    double shock_xpos = 0.5;
    bool shock_xpos_set = false;   // --shock_xpos: a fixed plane instead of the located shock
    bool conf_in_config_dir = true;
};

bool truthy(const std::string &v) {
    return v == "1" || v == ".true." || v == "true" || v == "T" || v == ".TRUE.";
}

// Switch table: long and short names of the reference's CLI (and a few of
// the engine's own, long names only).
int parse(int argc, char **argv, Options &o) {
    std::map<std::string, std::string> alias = {
        {"-dm", "--dir_mhd_data"}, {"-mc", "--mhd_config_filename"}, {"-nm", "--nptl_max"},
        {"-np", "--nptl"}, {"-ti", "--time_interp_flag"}, {"-dt", "--tinterval"},
        {"-ts", "--tstart"}, {"-te", "--tend"}, {"-tm", "--tmax_mhd"},
        {"-st", "--single_time_frame"}, {"-df", "--dist_flag"}, {"-pi", "--power_index"},
        {"-sf", "--split_flag"}, {"-sr", "--split_ratio"}, {"-ps", "--pmin_split"},
        {"-ni", "--nsteps_interval"}, {"-dd", "--diagnostics_directory"},
        {"-is", "--inject_at_shock"}, {"-in", "--inject_new_ptl"}, {"-tti", "--tmax_to_inject"},
        {"-ip", "--inject_part_box"}, {"-xs", "--ptl_xmin"}, {"-xe", "--ptl_xmax"},
        {"-ys", "--ptl_ymin"}, {"-ye", "--ptl_ymax"}, {"-zs", "--ptl_zmin"}, {"-ze", "--ptl_zmax"},
        {"-cf", "--conf_file"}, {"-nf", "--num_fine_steps"}, {"-nd", "--ndim_field"},
        {"-dp1", "--drift_param1"}, {"-dp2", "--drift_param2"}, {"-ch", "--charge"},
        {"-pv", "--particle_v0"}, {"-cd", "--check_drift_2d"}, {"-sc", "--spherical_coord"},
        {"-ug", "--uniform_grid"}, {"-i3", "--include_3rd_dim"}, {"-as", "--acc_by_surface"},
        {"-sf1", "--surface_filename1"}, {"-sn1", "--surface_norm1"},
        {"-s2e", "--surface2_existed"}, {"-ii", "--is_intersection"},
        {"-sf2", "--surface_filename2"}, {"-sn2", "--surface_norm2"}, {"-ft", "--focused_transport"},
        {"-nl", "--nlgc"}, {"-kk", "--kperp_kpara"}, {"-du", "--duu_init"},
        {"-pd", "--particle_data_dump"}, {"-ded", "--dump_escaped_dist"},
        {"-de", "--dump_escaped"}, {"-dw", "--dpp_wave"}, {"-ds", "--dpp_shear"},
        {"-ws", "--weak_scattering"}, {"-t0", "--tau0_scattering"},
        {"-ij", "--inject_large_jz"}, {"-iaj", "--inject_large_absj"},
        {"-ib", "--inject_large_db2"}, {"-iv", "--inject_large_divv"},
        {"-ir", "--inject_large_rho"}, {"-sn", "--inject_same_nptl"}, {"-jz", "--jz_min"},
        {"-ajm", "--absj_min"}, {"-dv", "--divv_min"}, {"-rm", "--rho_min"},
        {"-nn", "--ncells_large_jz_norm"}, {"-naj", "--ncells_large_absj_norm"},
        {"-nv", "--ncells_large_divv_norm"}, {"-nr", "--ncells_large_rho_norm"},
        {"-db2", "--db2_min"}, {"-nb", "--ncells_large_db2_norm"}, {"-db", "--deltab_flag"},
        {"-co", "--correlation"}, {"-tf", "--track_particle_flag"},
        {"-ptf", "--particle_tags_file"}, {"-vdt", "--varying_dt_mhd"},
        {"-rf", "--restart_flag"}, {"-qh", "--quota_hour"}, {"-ld", "--local_dist"},
        {"-sm", "--size_mpi_sub"}};
    for (int i = 1; i < argc; ++i) {
        std::string k = argv[i];
        if (alias.count(k)) k = alias[k];
        if (k == "--help" || k == "-h") return 1;
        if (i + 1 >= argc) { std::fprintf(stderr, "gpat_run: %s needs a value\n", argv[i]); return 2; }
        const std::string v = argv[++i];
        const double d = std::atof(v.c_str());
        if (k == "--dir_mhd_data") o.dir_mhd_data = v;
        else if (k == "--mhd_config_filename") o.mhd_config_filename = v;
        else if (k == "--nptl_max") o.nptl_max = (long long)d;
        else if (k == "--nptl") o.nptl = (long long)d;
        else if (k == "--time_interp_flag") o.time_interp_flag = (int)d;
        else if (k == "--tinterval") o.tinterval = d;
        else if (k == "--tstart") o.t_start = (int)d;
        else if (k == "--tend") o.t_end = (int)d;
        else if (k == "--tmax_mhd") o.tmax_mhd = (int)d;
        else if (k == "--single_time_frame") o.single_time_frame = (int)d;
        else if (k == "--dist_flag") o.dist_flag = (int)d;
        else if (k == "--power_index") o.power_index = d;
        else if (k == "--split_flag") o.split_flag = (int)d;
        else if (k == "--split_ratio") o.split_ratio = d;
        else if (k == "--pmin_split") o.pmin_split = d;
        else if (k == "--nsteps_interval") o.nsteps_interval = (int)d;
        else if (k == "--diagnostics_directory") o.diagnostics_directory = v;
        else if (k == "--inject_at_shock") o.inject_at_shock = truthy(v);
        else if (k == "--inject_new_ptl") o.inject_new_ptl = truthy(v);
        else if (k == "--tmax_to_inject") o.tmax_to_inject = (int)d;
        else if (k == "--inject_part_box") o.inject_part_box = truthy(v);
        else if (k == "--ptl_xmin") o.ptl_box[0] = d;
        else if (k == "--ptl_ymin") o.ptl_box[1] = d;
        else if (k == "--ptl_zmin") o.ptl_box[2] = d;
        else if (k == "--ptl_xmax") o.ptl_box[3] = d;
        else if (k == "--ptl_ymax") o.ptl_box[4] = d;
        else if (k == "--ptl_zmax") o.ptl_box[5] = d;
        else if (k == "--conf_file") o.conf_file = v;
        else if (k == "--num_fine_steps") o.num_fine_steps = (int)d;
        else if (k == "--ndim_field") o.ndim_field = (int)d;
        else if (k == "--drift_param1") o.drift_param1 = d;
        else if (k == "--drift_param2") o.drift_param2 = d;
        else if (k == "--charge") o.charge = (int)d;
        else if (k == "--particle_v0") o.particle_v0 = d;
        else if (k == "--check_drift_2d") o.check_drift_2d = (int)d;
        else if (k == "--spherical_coord") o.spherical_coord = (int)d;
        else if (k == "--uniform_grid") o.uniform_grid = (int)d;
        else if (k == "--include_3rd_dim") o.include_3rd_dim = (int)d;
        else if (k == "--acc_by_surface") o.acc_by_surface = (int)d;
        else if (k == "--surface_filename1") o.surface_filename1 = v;
        else if (k == "--surface_norm1") o.surface_norm1 = v;
        else if (k == "--surface2_existed") o.surface2_existed = truthy(v);
        else if (k == "--is_intersection") o.is_intersection = truthy(v);
        else if (k == "--surface_filename2") o.surface_filename2 = v;
        else if (k == "--surface_norm2") o.surface_norm2 = v;
        else if (k == "--focused_transport") o.focused_transport = truthy(v);
        else if (k == "--nlgc") o.nlgc = truthy(v);
        else if (k == "--kperp_kpara") o.kperp_kpara = d;
        else if (k == "--duu_init") o.duu_init = d;
        else if (k == "--particle_data_dump") o.particle_data_dump = (int)d;
        else if (k == "--dump_escaped_dist") o.dump_escaped_dist = truthy(v);
        else if (k == "--dump_escaped") o.dump_escaped = truthy(v);
        else if (k == "--dpp_wave") o.dpp_wave = (int)d;
        else if (k == "--dpp_shear") o.dpp_shear = (int)d;
        else if (k == "--weak_scattering") o.weak_scattering = (int)d;
        else if (k == "--tau0_scattering") o.tau0_scattering = d;
        else if (k == "--inject_large_jz") o.inject_large_jz = truthy(v);
        else if (k == "--inject_large_absj") o.inject_large_absj = truthy(v);
        else if (k == "--inject_large_db2") o.inject_large_db2 = truthy(v);
        else if (k == "--inject_large_divv") o.inject_large_divv = truthy(v);
        else if (k == "--inject_large_rho") o.inject_large_rho = truthy(v);
        else if (k == "--inject_same_nptl") o.inject_same_nptl = truthy(v);
        else if (k == "--jz_min") o.jz_min = d;
        else if (k == "--absj_min") o.absj_min = d;
        else if (k == "--divv_min") o.divv_min = d;
        else if (k == "--rho_min") o.rho_min = d;
        else if (k == "--ncells_large_jz_norm") o.ncells_large_jz_norm = (long long)d;
        else if (k == "--ncells_large_absj_norm") o.ncells_large_absj_norm = (long long)d;
        else if (k == "--ncells_large_divv_norm") o.ncells_large_divv_norm = (long long)d;
        else if (k == "--ncells_large_rho_norm") o.ncells_large_rho_norm = (long long)d;
        else if (k == "--db2_min") o.db2_min = d;
        else if (k == "--ncells_large_db2_norm") o.ncells_large_db2_norm = (long long)d;
        else if (k == "--deltab_flag") o.deltab_flag = (int)d;
        else if (k == "--correlation") o.correlation_flag = (int)d;
        else if (k == "--track_particle_flag") o.track_particle_flag = truthy(v);
        else if (k == "--particle_tags_file") o.particle_tags_file = v;
        else if (k == "--varying_dt_mhd") o.varying_dt_mhd = truthy(v);
        else if (k == "--restart_flag") o.restart_flag = truthy(v);
        else if (k == "--quota_hour") o.quota_hour = d;
        else if (k == "--local_dist") o.local_dist = truthy(v);
        else if (k == "--size_mpi_sub") o.size_mpi_sub = (int)d;
        else if (k == "--precision") {
            o.precision = (v == "fp64" || v == "0") ? GPAT_PREC_FP64 : GPAT_PREC_MIXED;
            o.precision_set = true;
        }
        else if (k == "--noise") o.noise = (v == "gauss" || v == "1") ? GPAT_NOISE_GAUSS : GPAT_NOISE_UNIFORM;
        else if (k == "--seed") o.seed = std::strtoull(v.c_str(), nullptr, 0);
        else if (k == "--device") o.device = (int)d;
        else if (k == "--bin_interval") o.bin_interval = (int)d;
        else if (k == "--shock_xpos") { o.shock_xpos = d; o.shock_xpos_set = true; }
        else if (k == "--conf_path_is_literal") o.conf_in_config_dir = !truthy(v);
        else { std::fprintf(stderr, "gpat_run: unknown switch %s\n", argv[i - 1]); return 2; }
    }
    return 0;
}

#define CHECK(call)                                                                    \
    do {                                                                               \
        int rc_ = (call);                                                              \
        if (rc_ != GPAT_OK && rc_ != GPAT_ERR_CAPACITY) {                              \
            std::fprintf(stderr, "gpat_run: %s failed (%d): %s\n", #call, rc_,         \
                         h ? gpat_last_error(h) : "");                                 \
            if (h) gpat_destroy(h);                                                    \
            return 1;                                                                  \
        }                                                                              \
    } while (0)

// dump_particles (diagnostics.f90:1810-1888) without HDF5.  The file holds
// int64 nptl and then the datasets of particles_XXXX.h5 in the reference's
// order, nptl values each: x y z p v mu weight t dt (float64), split_times
// count_flag (int8), origin nsteps_tracked nsteps_pushed tag_injected
// tag_splitted (int32).
// particles_XXXX.dat (dump_particles), or escaped_particles_XXXX.dat
// (dump_escaped_particles, diagnostics.f90:1896-1978) when escaped.
int write_particles(gpat_handle_t *h, const std::string &dir, int frame, bool escaped = false) {
    int64_t n = 0;
    int rc;
    if (escaped) {
        gpat_particles_t none;
        std::memset(&none, 0, sizeof none);
        rc = gpat_get_escaped_particles(h, &none, 0, &n);
        if (rc && rc != GPAT_ERR_CAPACITY) return rc;
    } else {
        gpat_counters_t c;
        rc = gpat_get_counters(h, &c);
        if (rc) return rc;
        n = c.nptl_current;
    }
    const size_t m = (size_t)(n > 0 ? n : 1);
    std::vector<double> f64[9];
    std::vector<int8_t> i8[2];
    std::vector<int32_t> i32[5];
    std::vector<uint32_t> ctr(m);
    for (auto &v : f64) v.resize(m);
    for (auto &v : i8) v.resize(m);
    for (auto &v : i32) v.resize(m);
    gpat_particles_t P;
    P.x = f64[0].data(); P.y = f64[1].data(); P.z = f64[2].data(); P.p = f64[3].data();
    P.v = f64[4].data(); P.mu = f64[5].data(); P.weight = f64[6].data(); P.t = f64[7].data();
    P.dt = f64[8].data();
    P.split_times = i8[0].data(); P.count_flag = i8[1].data();
    P.origin = i32[0].data(); P.nsteps_tracked = i32[1].data(); P.nsteps_pushed = i32[2].data();
    P.tag_injected = i32[3].data(); P.tag_splitted = i32[4].data();
    P.rng_ctr = ctr.data();
    int64_t got = 0;
    rc = escaped ? gpat_get_escaped_particles(h, &P, n, &got) : gpat_get_particles(h, &P, n, &got);
    if (rc) return rc;
    char name[64];
    std::snprintf(name, sizeof name, escaped ? "escaped_particles_%04d.dat" : "particles_%04d.dat",
                  frame);
    FILE *f = std::fopen((dir + name).c_str(), "wb");
    if (!f) return GPAT_ERR_IO;
    bool ok = std::fwrite(&got, 8, 1, f) == 1;
    for (auto &v : f64) ok = ok && std::fwrite(v.data(), 8, (size_t)got, f) == (size_t)got;
    for (auto &v : i8) ok = ok && std::fwrite(v.data(), 1, (size_t)got, f) == (size_t)got;
    for (auto &v : i32) ok = ok && std::fwrite(v.data(), 4, (size_t)got, f) == (size_t)got;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GPAT_OK : GPAT_ERR_IO;
}

// dump_tracked_particles (particle_module.f90:6235-6299) without HDF5:
// int64 nsteps_tracking_max, int64 nptl_tracking, then the datasets of
// particles_tracked_XXXX.h5 in the reference's order, each
// particles_tracked(nsteps_tracking_max, nptl_tracking) in Fortran order:
// x y z p v mu weight t dt (float64), split_times count_flag (int8), origin
// nsteps_tracked nsteps_pushed tag_injected tag_splitted (int32).
int write_tracked(gpat_handle_t *h, const std::string &dir, int frame) {
    int64_t nsteps = 0, dropped = 0;
    int32_t ntrk = 0;
    int rc = gpat_tracking_dims(h, &nsteps, &ntrk, &dropped);
    if (rc) return rc;
    const size_t m = (size_t)nsteps * (size_t)ntrk;
    std::vector<double> f64[9];
    std::vector<int8_t> i8[2];
    std::vector<int32_t> i32[5];
    for (auto &v : f64) v.resize(m);
    for (auto &v : i8) v.resize(m);
    for (auto &v : i32) v.resize(m);
    gpat_particles_t P;
    P.x = f64[0].data(); P.y = f64[1].data(); P.z = f64[2].data(); P.p = f64[3].data();
    P.v = f64[4].data(); P.mu = f64[5].data(); P.weight = f64[6].data(); P.t = f64[7].data();
    P.dt = f64[8].data();
    P.split_times = i8[0].data(); P.count_flag = i8[1].data();
    P.origin = i32[0].data(); P.nsteps_tracked = i32[1].data(); P.nsteps_pushed = i32[2].data();
    P.tag_injected = i32[3].data(); P.tag_splitted = i32[4].data();
    P.rng_ctr = nullptr;
    rc = gpat_get_tracked_particles(h, &P);
    if (rc) return rc;
    char name[64];
    std::snprintf(name, sizeof name, "particles_tracked_%04d.dat", frame);
    FILE *f = std::fopen((dir + name).c_str(), "wb");
    if (!f) return GPAT_ERR_IO;
    const int64_t dims[2] = {nsteps, (int64_t)ntrk};
    bool ok = std::fwrite(dims, 8, 2, f) == 2;
    for (auto &v : f64) ok = ok && std::fwrite(v.data(), 8, m, f) == m;
    for (auto &v : i8) ok = ok && std::fwrite(v.data(), 1, m, f) == m;
    for (auto &v : i32) ok = ok && std::fwrite(v.data(), 4, m, f) == m;
    ok = (std::fclose(f) == 0) && ok;
    if (dropped)
        std::fprintf(stderr, "gpat_run: %lld tracked records past nsteps_tracking_max dropped\n",
                     (long long)dropped);
    return ok ? GPAT_OK : GPAT_ERR_IO;
}

// read_particles for a restart: particles_XXXX.dat as write_particles makes
// it, with the Philox counters of prng_state_XXXX.dat when present (they
// take the place of the MT19937 states of save_prng / init_prng).
int read_particles(gpat_handle_t *h, const std::string &dir, int frame) {
    char name[64];
    std::snprintf(name, sizeof name, "particles_%04d.dat", frame);
    FILE *f = std::fopen((dir + name).c_str(), "rb");
    if (!f) return GPAT_ERR_IO;
    int64_t n = 0;
    bool ok = std::fread(&n, 8, 1, f) == 1 && n >= 0;
    const size_t m = (size_t)(ok && n > 0 ? n : 1);
    std::vector<double> f64[9];
    std::vector<int8_t> i8[2];
    std::vector<int32_t> i32[5];
    std::vector<uint32_t> ctr(m, 0u);
    for (auto &v : f64) { v.resize(m); if (ok) ok = std::fread(v.data(), 8, (size_t)n, f) == (size_t)n; }
    for (auto &v : i8) { v.resize(m); if (ok) ok = std::fread(v.data(), 1, (size_t)n, f) == (size_t)n; }
    for (auto &v : i32) { v.resize(m); if (ok) ok = std::fread(v.data(), 4, (size_t)n, f) == (size_t)n; }
    std::fclose(f);
    if (!ok) return GPAT_ERR_IO;
    std::snprintf(name, sizeof name, "prng_state_%04d.dat", frame);
    if (FILE *g = std::fopen((dir + name).c_str(), "rb")) {
        int64_t nc = 0;
        ok = std::fread(&nc, 8, 1, g) == 1 && nc == n &&
             std::fread(ctr.data(), 4, (size_t)n, g) == (size_t)n;
        std::fclose(g);
        if (!ok) return GPAT_ERR_IO;
    }
    gpat_particles_t P;
    P.x = f64[0].data(); P.y = f64[1].data(); P.z = f64[2].data(); P.p = f64[3].data();
    P.v = f64[4].data(); P.mu = f64[5].data(); P.weight = f64[6].data(); P.t = f64[7].data();
    P.dt = f64[8].data();
    P.split_times = i8[0].data(); P.count_flag = i8[1].data();
    P.origin = i32[0].data(); P.nsteps_tracked = i32[1].data(); P.nsteps_pushed = i32[2].data();
    P.tag_injected = i32[3].data(); P.tag_splitted = i32[4].data();
    P.rng_ctr = ctr.data();
    return gpat_put_particles(h, &P, n);
}

// prng_state_XXXX.dat: int64 nptl, then the particles' Philox counters in
// the order of particles_XXXX.dat.
int write_prng_state(gpat_handle_t *h, const std::string &dir, int frame) {
    gpat_counters_t c;
    int rc = gpat_get_counters(h, &c);
    if (rc) return rc;
    const int64_t n = c.nptl_current;
    std::vector<uint32_t> ctr((size_t)(n > 0 ? n : 1));
    gpat_particles_t P;
    std::memset(&P, 0, sizeof P);
    P.rng_ctr = ctr.data();
    int64_t got = 0;
    rc = gpat_get_particles(h, &P, n, &got);
    if (rc) return rc;
    char name[64];
    std::snprintf(name, sizeof name, "prng_state_%04d.dat", frame);
    FILE *f = std::fopen((dir + name).c_str(), "wb");
    if (!f) return GPAT_ERR_IO;
    bool ok = std::fwrite(&got, 8, 1, f) == 1 &&
              std::fwrite(ctr.data(), 4, (size_t)got, f) == (size_t)got;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GPAT_OK : GPAT_ERR_IO;
}

// save_particle_module_state / read_particle_module_state
// (particle_module.f90:5532-5660) for one rank without HDF5:
// particle_module_state_XXXX.dat holds int64 nptl_current, nptl_split,
// tag_max, float64 leak, leak_negp, then the exact fixed-point sums
// (uint64 leak_hi, leak_lo, leak_negp_hi, leak_negp_lo).
int write_module_state(gpat_handle_t *h, const std::string &dir, int frame) {
    gpat_counters_t c;
    int rc = gpat_get_counters(h, &c);
    if (rc) return rc;
    char name[64];
    std::snprintf(name, sizeof name, "particle_module_state_%04d.dat", frame);
    FILE *f = std::fopen((dir + name).c_str(), "wb");
    if (!f) return GPAT_ERR_IO;
    const int64_t i3[3] = {c.nptl_current, c.nptl_split, c.tag_max};
    const double d2[2] = {c.leak, c.leak_negp};
    const uint64_t u4[4] = {c.leak_hi, c.leak_lo, c.leak_negp_hi, c.leak_negp_lo};
    bool ok = std::fwrite(i3, 8, 3, f) == 3 && std::fwrite(d2, 8, 2, f) == 2 &&
              std::fwrite(u4, 8, 4, f) == 4;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GPAT_OK : GPAT_ERR_IO;
}

int read_module_state(gpat_handle_t *h, const std::string &dir, int frame) {
    char name[64];
    std::snprintf(name, sizeof name, "particle_module_state_%04d.dat", frame);
    FILE *f = std::fopen((dir + name).c_str(), "rb");
    if (!f) return GPAT_ERR_IO;
    int64_t i3[3];
    double d2[2];
    uint64_t u4[4];
    bool ok = std::fread(i3, 8, 3, f) == 3 && std::fread(d2, 8, 2, f) == 2 &&
              std::fread(u4, 8, 4, f) == 4;
    std::fclose(f);
    if (!ok) return GPAT_ERR_IO;
    gpat_counters_t c;
    int rc = gpat_get_counters(h, &c);
    if (rc) return rc;
    c.nptl_split = i3[1];
    c.tag_max = i3[2];
    c.leak = d2[0];
    c.leak_negp = d2[1];
    c.leak_hi = u4[0]; c.leak_lo = u4[1]; c.leak_negp_hi = u4[2]; c.leak_negp_lo = u4[3];
    return gpat_set_counters(h, &c);
}

std::string frame_name(const std::string &dir, int tf) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "mhd_data_%04d", tf);
    return dir + buf;
}

}  // namespace

int main(int argc, char **argv) {
    Options o;
    const int prc = parse(argc, argv, o);
    if (prc) {
        std::fprintf(stderr, "usage: gpat_run [reference switches] (see stochastic-mhd.f90)\n");
        return prc == 1 ? 0 : 2;
    }
    if (o.single_time_frame == 1) o.time_interp_flag = 0;   // stochastic-mhd.f90:134-136
    if (o.size_mpi_sub != 1) {
        std::fprintf(stderr, "gpat_run: one rank per device; -sm must be 1\n");
        return 2;
    }
    if (o.inject_large_db2 && o.deltab_flag != 1) {
        std::fprintf(stderr, "gpat_run: -ib needs -db 1 (the magnetic-fluctuation arrays)\n");
        return 2;
    }
    // Options the split-precision mover does not have (focused transport,
    // Dpp, turbulence arrays, spherical or non-uniform grids, include_3rd_dim,
    // surfaces, tracking, 1D) run on the FP64 mover unless asked otherwise.
    if ((o.focused_transport || o.dpp_wave || o.dpp_shear || o.deltab_flag ||
         o.correlation_flag || o.spherical_coord == 1 || o.uniform_grid != 1 ||
         o.include_3rd_dim == 1 || o.acc_by_surface == 1 || o.track_particle_flag ||
         o.ndim_field == 1) &&
        !o.precision_set)
        o.precision = GPAT_PREC_FP64;
    gpat_handle_t *h = nullptr;

    gpat_mhd_config_t cfg;
    const std::string cfg_path = o.dir_mhd_data + o.mhd_config_filename;
    CHECK(gpat_load_mhd_config(cfg_path.c_str(), &cfg));

    gpat_params_t p;
    std::memset(&p, 0, sizeof p);
    p.npp_global = 128;
    const std::string conf = o.conf_in_config_dir ? "config/" + o.conf_file : o.conf_file;
    CHECK(gpat_read_particle_params(conf.c_str(), &p));
    p.drift1 = o.drift_param1;
    p.drift2 = o.drift_param2;
    p.charge = o.charge;
    p.check_drift_2d = o.check_drift_2d;
    p.ndim = o.ndim_field;
    p.seed = o.seed;
    p.noise = o.noise;
    p.precision = o.precision;
    p.nptl_max = o.nptl_max;
    p.time_interp = o.time_interp_flag;
    p.bin_interval = o.bin_interval;
    p.duu0 = o.duu_init;
    p.dpp_wave = o.dpp_wave;
    p.dpp_shear = o.dpp_shear;
    p.weak_scattering = o.weak_scattering;
    p.tau0 = o.tau0_scattering;
    p.deltab_flag = o.deltab_flag;
    p.correlation_flag = o.correlation_flag;
    // set_mhd_grid_type (:179)
    p.spherical_coord = o.spherical_coord == 1 ? 1 : 0;
    p.nonuniform_grid = o.uniform_grid == 1 ? 0 : 1;
    p.include_3rd_dim = (o.include_3rd_dim == 1 && o.ndim_field == 2) ? 1 : 0;
    CHECK(gpat_create(&p, &cfg, o.device, &h));
    // set_local_grid_positions (:186): xpos.dat, ypos.dat, zpos.dat
    if (p.nonuniform_grid) CHECK(gpat_read_grid_positions(h, o.dir_mhd_data.c_str()));
    // init_acc_surface (:196-203)
    if (o.acc_by_surface == 1)
        CHECK(gpat_init_acc_surface(h, o.surface_norm1.c_str(),
                                    o.surface2_existed ? o.surface_norm2.c_str() : nullptr,
                                    o.is_intersection ? 1 : 0));
    const auto wall_start = std::chrono::steady_clock::now();
    // the time stamps of the MHD frames (stochastic-mhd.f90:173-178)
    if (o.varying_dt_mhd)
        CHECK(gpat_load_tstamps_mhd(h, o.t_start, o.t_end, o.tmax_mhd, o.dir_mhd_data.c_str()));
    else
        CHECK(gpat_calc_tstamps_mhd(h, o.t_start, o.t_end));
    // restart (stochastic-mhd.f90:224-238): the frame of restart/latest_restart,
    // its particles and module state
    const std::string restart = o.diagnostics_directory + "restart/";
    int tmin = o.t_start;
    if (o.restart_flag) {
        FILE *lr = std::fopen((restart + "latest_restart").c_str(), "rb");
        int32_t t32 = 0;
        const bool got = lr && std::fread(&t32, 4, 1, lr) == 1;
        if (lr) std::fclose(lr);
        if (!got) {
            std::fprintf(stderr, "gpat_run: cannot read %slatest_restart\n", restart.c_str());
            gpat_destroy(h);
            return 1;
        }
        tmin = t32;
        CHECK(read_particles(h, restart, tmin));
        CHECK(read_module_state(h, restart, tmin));
    }
    // init_particle_tracking (stochastic-mhd.f90:241-244)
    const std::string track_dir = o.diagnostics_directory + "particle_tracking/";
    if (o.track_particle_flag)
        CHECK(gpat_read_particle_tracking(h, (track_dir + o.particle_tags_file).c_str(),
                                          o.nsteps_interval));

    // Frame tmin into farray1, gradients (:321, :350).
    CHECK(gpat_read_field_data(h, frame_name(o.dir_mhd_data, tmin).c_str(), 0));
    // read_acc_surface of <dir><surface_filename>_XXXX.dat (:324-333, :406-415)
    auto read_surfaces = [&](int tf, int var_flag) -> int {
        if (o.acc_by_surface != 1) return GPAT_OK;
        char num[16];
        std::snprintf(num, sizeof num, "_%04d.dat", tf);
        const std::string f1 = o.dir_mhd_data + o.surface_filename1 + num;
        const std::string f2 = o.dir_mhd_data + o.surface_filename2 + num;
        return gpat_read_acc_surface(h, var_flag, f1.c_str(),
                                     o.surface2_existed ? f2.c_str() : nullptr);
    };
    auto read_turbulence = [&](int tf, int var_flag) -> int {
        char num[16];
        std::snprintf(num, sizeof num, "%04d", tf);
        if (o.deltab_flag == 1) {   // stochastic-mhd.f90:337-346, :417-424
            int rc = gpat_read_magnetic_fluctuation(h, (o.dir_mhd_data + "deltab_" + num).c_str(),
                                                    var_flag);
            if (rc) return rc;
        }
        if (o.correlation_flag == 1)
            return gpat_read_correlation_length(h, (o.dir_mhd_data + "lc_" + num).c_str(), var_flag);
        return GPAT_OK;
    };
    CHECK(read_surfaces(tmin, 0));
    CHECK(read_turbulence(tmin, 0));
    CHECK(gpat_calc_fields_gradients(h, 0));
    double part_box[6];
    if (o.inject_part_box) {
        for (int i = 0; i < 6; ++i) part_box[i] = o.ptl_box[i];
    } else {
        part_box[0] = cfg.xmin; part_box[1] = cfg.ymin; part_box[2] = cfg.zmin;
        part_box[3] = cfg.xmin + cfg.nx * cfg.dx; part_box[4] = cfg.ymin + cfg.ny * cfg.dy;
        part_box[5] = o.ndim_field == 3 ? cfg.zmin + cfg.nz * cfg.dz : cfg.zmax;
    }

    const int npp = p.npp_global;
    std::vector<double> edges(npp + 1), fglobal(npp);
    std::vector<uint64_t> counts(npp);
    CHECK(gpat_pbins_edges(h, edges.data()));
    const std::string qpath = o.diagnostics_directory + "quick.dat";
    FILE *quick = std::fopen(qpath.c_str(), o.restart_flag ? "a" : "w");
    if (!quick) { std::fprintf(stderr, "gpat_run: cannot write %s\n", qpath.c_str()); gpat_destroy(h); return 1; }
    if (!o.restart_flag)
        std::fprintf(quick, "%6s%13s%13s%13s%13s%13s%13s%13s%13s\n", "iframe", "nptl_current",
                     "nptl_split", "ntot", "leak", "leak_negp", "pdt_min", "pdt_max", "pdt_avg");

    // read_diagnostics_params (diagnostics.f90:2049-2222): local-distribution
    // set k is on when dump_intervalk < t_end - t_start; mu bins only with
    // focused transport.
    struct LocalSet { int k; gpat_local_dist_t spec; };
    std::vector<LocalSet> local_sets;
    if (o.local_dist) {
        auto var = [&](const std::string &key) -> double {
            double v = -1.0;
            return gpat_get_variable(conf.c_str(), key.c_str(), &v) == GPAT_OK ? v : -1.0;
        };
        for (int k = 1; k <= 4; ++k) {
            const std::string s = std::to_string(k);
            if (!((int)var("dump_interval" + s) < o.t_end - o.t_start)) continue;
            gpat_local_dist_t sp;
            std::memset(&sp, 0, sizeof sp);
            sp.pmin = var("pmin" + s);
            sp.pmax = var("pmax" + s);
            sp.npbins = (int)var("npbins" + s);
            sp.nmu = o.focused_transport ? (int)var("nmu" + s) : 1;
            sp.rx = (int)var("rx" + s);
            sp.ry = (int)var("ry" + s);
            sp.rz = (int)var("rz" + s);
            if (!(sp.pmin > 0.0 && sp.pmax > sp.pmin) || sp.npbins < 1 || sp.nmu < 1 ||
                sp.rx < 1 || sp.ry < 1 || sp.rz < 1) {
                std::fprintf(stderr, "gpat_run: local distribution %d: bad or missing "
                             "pmin/pmax/npbins/nmu/rx/ry/rz in %s\n", k, conf.c_str());
                gpat_destroy(h);
                return 2;
            }
            local_sets.push_back({k, sp});
        }
    }
    // flocalK_XXXX.dat: int32 {nmu, npbins, nrx, nry, nrz}, the npbins + 1
    // p edges and nmu + 1 mu edges (pbinsK_edges, mubinsK_edges), flocalK
    // in Fortran order, then the uint64 particle counts.
    auto write_local = [&](int frame) -> int {
        for (const LocalSet &ls : local_sets) {
            int32_t dims[5];
            int rc = gpat_local_distribution_dims(h, &ls.spec, dims);
            if (rc) return rc;
            const size_t nb = (size_t)dims[0] * dims[1] * dims[2] * dims[3] * dims[4];
            std::vector<double> fl(nb);
            std::vector<uint64_t> cl(nb);
            rc = gpat_calc_local_distribution(h, &ls.spec, fl.data(), cl.data());
            if (rc) return rc;
            // init_local_particle_distributions (:262-290)
            const double lo = std::log10(ls.spec.pmin), hi = std::log10(ls.spec.pmax);
            const double dlog = (hi - lo) / ls.spec.npbins;
            const double dmu = (double)(2.0f / (float)ls.spec.nmu);
            std::vector<double> pe(ls.spec.npbins + 1), me(ls.spec.nmu + 1);
            for (int i = 0; i <= ls.spec.npbins; ++i) pe[i] = std::pow(10.0, lo + i * dlog);
            for (int i = 0; i <= ls.spec.nmu; ++i) me[i] = -1.0 + i * dmu;
            char name[64];
            std::snprintf(name, sizeof name, "flocal%d_%04d.dat", ls.k, frame);
            FILE *f = std::fopen((o.diagnostics_directory + name).c_str(), "wb");
            if (!f) return GPAT_ERR_IO;
            bool ok = std::fwrite(dims, 4, 5, f) == 5 &&
                      std::fwrite(pe.data(), 8, pe.size(), f) == pe.size() &&
                      std::fwrite(me.data(), 8, me.size(), f) == me.size() &&
                      std::fwrite(fl.data(), 8, nb, f) == nb &&
                      std::fwrite(cl.data(), 8, nb, f) == nb;
            ok = (std::fclose(f) == 0) && ok;
            if (!ok) return GPAT_ERR_IO;
        }
        return GPAT_OK;
    };
    // With focused transport the global and escaped distributions carry
    // nmu_global pitch-angle bins (read_diagnostics_params :2105-2111):
    // fglobal_mu_XXXX.dat / fescaped_mu_XXXX.dat hold int32 nmu, npp, nface
    // (1 for fglobal), the nmu + 1 mu edges, the npp + 1 p edges, the
    // weights (nmu, npp, nface) in Fortran order and the uint64 counts.
    int nmu_global = 1;
    if (o.focused_transport) {
        double v = -1.0;
        if (gpat_get_variable(conf.c_str(), "nmu_global", &v) == GPAT_OK && v >= 1.0)
            nmu_global = (int)v;
    }
    auto write_mu = [&](const char *stem, int frame, bool escaped) -> int {
        const int nface = escaped ? 2 * o.ndim_field : 1;
        const size_t nb = (size_t)nmu_global * npp * nface;
        std::vector<double> fm(nb);
        std::vector<uint64_t> cm(nb);
        int rc = escaped ? gpat_calc_escaped_distributions_mu(h, nmu_global, fm.data(), cm.data())
                         : gpat_calc_particle_distributions_mu(h, nmu_global, fm.data(), cm.data());
        if (rc) return rc;
        const double dmu = (double)(2.0f / (float)nmu_global);
        std::vector<double> me(nmu_global + 1);
        for (int i = 0; i <= nmu_global; ++i) me[i] = -1.0 + i * dmu;
        char name[64];
        std::snprintf(name, sizeof name, "%s_%04d.dat", stem, frame);
        FILE *f = std::fopen((o.diagnostics_directory + name).c_str(), "wb");
        if (!f) return GPAT_ERR_IO;
        const int32_t hdr[3] = {nmu_global, npp, nface};
        bool ok = std::fwrite(hdr, 4, 3, f) == 3 &&
                  std::fwrite(me.data(), 8, me.size(), f) == me.size() &&
                  std::fwrite(edges.data(), 8, edges.size(), f) == edges.size() &&
                  std::fwrite(fm.data(), 8, nb, f) == nb && std::fwrite(cm.data(), 8, nb, f) == nb;
        ok = (std::fclose(f) == 0) && ok;
        return ok ? GPAT_OK : GPAT_ERR_IO;
    };
    // save_local_escaped_distributions (diagnostics.f90:1536-1600):
    // fescapedK_XXXX.dat holds int32 {nmu, npbins, nrx, nry, nrz}, then for
    // the x faces (and y from 2D, z in 3D) the weights fescapedK_x(nmu,
    // npbins, nry, nrz, 2) etc. in Fortran order followed by their uint64
    // counts.
    auto write_local_escaped = [&](int frame) -> int {
        for (const LocalSet &ls : local_sets) {
            int32_t dims[5];
            int rc = gpat_local_distribution_dims(h, &ls.spec, dims);
            if (rc) return rc;
            const size_t mp = (size_t)dims[0] * dims[1];
            const size_t sz[3] = {mp * dims[3] * dims[4] * 2, mp * dims[2] * dims[4] * 2,
                                  mp * dims[2] * dims[3] * 2};
            std::vector<double> fv[3];
            std::vector<uint64_t> cv[3];
            for (int k = 0; k < o.ndim_field; ++k) { fv[k].resize(sz[k]); cv[k].resize(sz[k]); }
            auto dp = [&](int k) { return k < o.ndim_field ? fv[k].data() : nullptr; };
            auto up = [&](int k) { return k < o.ndim_field ? cv[k].data() : nullptr; };
            rc = gpat_calc_local_escaped_distribution(h, &ls.spec, dp(0), dp(1), dp(2), up(0),
                                                      up(1), up(2));
            if (rc) return rc;
            char name[64];
            std::snprintf(name, sizeof name, "fescaped%d_%04d.dat", ls.k, frame);
            FILE *f = std::fopen((o.diagnostics_directory + name).c_str(), "wb");
            if (!f) return GPAT_ERR_IO;
            bool ok = std::fwrite(dims, 4, 5, f) == 5;
            for (int k = 0; k < o.ndim_field; ++k)
                ok = ok && std::fwrite(fv[k].data(), 8, sz[k], f) == sz[k] &&
                     std::fwrite(cv[k].data(), 8, sz[k], f) == sz[k];
            ok = (std::fclose(f) == 0) && ok;
            if (!ok) return GPAT_ERR_IO;
        }
        return GPAT_OK;
    };
    // get_pmax_global (diagnostics.f90:1691-1721): pmax_global.dat, one
    // line per frame, created at the initial diagnostics
    auto write_pmax = [&](bool create) -> int {
        double pm = 0.0;
        int rc = gpat_get_pmax_global(h, &pm);
        if (rc) return rc;
        FILE *f = std::fopen((o.diagnostics_directory + "pmax_global.dat").c_str(),
                             create ? "w" : "a");
        if (!f) return GPAT_ERR_IO;
        std::fprintf(f, "%13.6E\n", pm);
        std::fclose(f);
        return GPAT_OK;
    };

    auto diagnostics = [&](int frame) -> int {
        double q[8];
        int rc = gpat_quick_check(h, q);
        if (rc) return rc;
        std::fprintf(quick, "%06d%13.6E%13.6E%13.6E%13.6E%13.6E%13.6E%13.6E%13.6E\n", frame, q[0],
                     q[1], q[2], q[3], q[4], q[5], q[6], q[7]);
        std::fflush(quick);
        rc = gpat_calc_particle_distributions(h, fglobal.data(), counts.data());
        if (rc) return rc;
        char name[64];
        std::snprintf(name, sizeof name, "fdists_%04d.dat", frame);
        FILE *f = std::fopen((o.diagnostics_directory + name).c_str(), "wb");
        if (!f) return GPAT_ERR_IO;
        const int32_t n32 = npp;
        std::fwrite(&n32, 4, 1, f);
        std::fwrite(edges.data(), 8, edges.size(), f);
        std::fwrite(fglobal.data(), 8, fglobal.size(), f);
        std::fwrite(counts.data(), 8, counts.size(), f);
        std::fclose(f);
        if (o.focused_transport) {
            const int rc = write_mu("fglobal_mu", frame, false);
            if (rc) return rc;
        }
        return write_local(frame);
    };

    // fescaped_XXXX.dat: int32 npp, int32 2 ndim, npp + 1 edges, the
    // weighted counts fescaped(npp, 2 ndim) (Fortran order), uint64 counts.
    auto write_escaped_dist = [&](int frame) -> int {
        const int ncol = 2 * o.ndim_field;
        std::vector<double> fe((size_t)npp * ncol);
        std::vector<uint64_t> ce((size_t)npp * ncol);
        int rc = gpat_calc_escaped_distributions(h, fe.data(), ce.data());
        if (rc) return rc;
        char name[64];
        std::snprintf(name, sizeof name, "fescaped_%04d.dat", frame);
        FILE *f = std::fopen((o.diagnostics_directory + name).c_str(), "wb");
        if (!f) return GPAT_ERR_IO;
        const int32_t hdr[2] = {npp, ncol};
        std::fwrite(hdr, 4, 2, f);
        std::fwrite(edges.data(), 8, edges.size(), f);
        std::fwrite(fe.data(), 8, fe.size(), f);
        std::fwrite(ce.data(), 8, ce.size(), f);
        std::fclose(f);
        if (o.focused_transport) {
            rc = write_mu("fescaped_mu", frame, true);
            if (rc) return rc;
        }
        return write_local_escaped(frame);
    };

    int tf_done = o.t_end;
    bool reached_quota = false;
    for (int tf = tmin + 1; tf <= o.t_end; ++tf) {
        if (o.single_time_frame == 0 && tf <= o.tmax_mhd) {
            CHECK(gpat_read_field_data(h, frame_name(o.dir_mhd_data, tf).c_str(), o.time_interp_flag));
            CHECK(read_surfaces(tf, o.time_interp_flag));
            CHECK(read_turbulence(tf, o.time_interp_flag));
            CHECK(gpat_calc_fields_gradients(h, o.time_interp_flag));
        }
        const int ct = tf - o.t_start;
        if (o.inject_at_shock) {
            // locate_shock_xpos + inject_particles_at_shock (:451-454), or a
            // fixed plane with --shock_xpos
            if (o.shock_xpos_set)
                CHECK(gpat_inject_particles_at_x(h, o.nptl, o.shock_xpos, o.tinterval,
                                                 o.dist_flag, o.particle_v0, ct, o.power_index));
            else
                CHECK(gpat_inject_particles_at_shock(h, o.nptl, o.tinterval, o.dist_flag,
                                                     o.particle_v0, ct, o.power_index));
        } else if ((tf == o.t_start + 1 || o.inject_new_ptl) && tf <= o.tmax_to_inject) {
            // stochastic-mhd.f90:455-483: the first large-quantity option set wins
            int quantity = -1;
            double qmin = 0.0;
            long long norm = 1;
            if (o.inject_large_jz) { quantity = GPAT_LARGE_JZ; qmin = o.jz_min; norm = o.ncells_large_jz_norm; }
            else if (o.inject_large_absj) { quantity = GPAT_LARGE_ABSJ; qmin = o.absj_min; norm = o.ncells_large_absj_norm; }
            else if (o.inject_large_db2) { quantity = GPAT_LARGE_DB2; qmin = o.db2_min; norm = o.ncells_large_db2_norm; }
            else if (o.inject_large_divv) { quantity = GPAT_LARGE_DIVV; qmin = o.divv_min; norm = o.ncells_large_divv_norm; }
            else if (o.inject_large_rho) { quantity = GPAT_LARGE_RHO; qmin = o.rho_min; norm = o.ncells_large_rho_norm; }
            if (quantity >= 0) {
                int64_t injected = 0;
                CHECK(gpat_inject_particles_at_large(h, quantity, o.nptl, o.tinterval, o.dist_flag,
                                                     o.particle_v0, ct, o.inject_same_nptl, qmin,
                                                     norm, part_box, o.power_index, &injected));
            } else {
                CHECK(gpat_inject_particles_spatial_uniform(h, o.nptl, o.tinterval, o.dist_flag,
                                                            o.particle_v0, ct, part_box,
                                                            o.power_index));
            }
        }
        // initial diagnostics unless tracking (:486-495)
        if (tf == o.t_start + 1 && !o.track_particle_flag) {
            CHECK(write_pmax(true));
            CHECK(diagnostics(o.t_start));
            if (o.particle_data_dump == 1) CHECK(write_particles(h, o.diagnostics_directory, o.t_start));
        }
        // a tracked run moves with one fine step (:498-504)
        CHECK(gpat_particle_mover(h, o.focused_transport, o.nlgc, o.kperp_kpara, o.nsteps_interval,
                                  ct, o.track_particle_flag ? 1 : o.num_fine_steps,
                                  o.dump_escaped_dist ? 1 : 0));
        if (o.track_particle_flag) CHECK(write_tracked(h, track_dir, tf));
        if (o.split_flag == 1) CHECK(gpat_split_particle(h, o.split_ratio, o.pmin_split, o.nsteps_interval));
        if (!o.track_particle_flag) {
            CHECK(write_pmax(false));
            CHECK(diagnostics(tf));
            if (o.particle_data_dump == 1) CHECK(write_particles(h, o.diagnostics_directory, tf));
            if (o.dump_escaped_dist) {
                // distributions_diagnostics' escaped distributions, then
                // dump_escaped_particles and reset_escaped_particles (:519-533)
                CHECK(write_escaped_dist(tf));
                if (o.dump_escaped) CHECK(write_particles(h, o.diagnostics_directory, tf, true));
                CHECK(gpat_reset_escaped_particles(h));
            }
        }
        if (o.time_interp_flag == 1) CHECK(gpat_copy_fields(h));
        gpat_counters_t c;
        CHECK(gpat_get_counters(h, &c));
        std::printf("frame %d: %lld particles, %llu pushes, mover %.2f ms\n", tf,
                    (long long)c.nptl_current, (unsigned long long)c.last_mover_steps,
                    c.last_mover_ms);
        // stop 30 minutes before the wall-time quota (:559-565)
        const double uptime = std::chrono::duration<double>(std::chrono::steady_clock::now() -
                                                            wall_start).count();
        if (uptime > (o.quota_hour - 0.5) * 3600.0) {
            reached_quota = true;
            tf_done = tf;
            break;
        }
    }
    std::fclose(quick);
    // Restart files (stochastic-mhd.f90:252-273): particles and module state
    // under t_end and latest_restart holding the last finished frame.  When
    // the quota stopped the loop early they are also written under that
    // frame, which is the one a restart reads.
    mkdir(restart.c_str(), 0755);
    if (reached_quota) std::printf("reached the quota time at frame %d\n", tf_done);
    for (int fr : {o.t_end, tf_done}) {
        CHECK(write_particles(h, restart, fr));
        CHECK(write_prng_state(h, restart, fr));
        CHECK(write_module_state(h, restart, fr));
        if (fr == tf_done) break;
    }
    {
        FILE *lr = std::fopen((restart + "latest_restart").c_str(), "wb");
        const int32_t t32 = tf_done;
        const bool ok = lr && std::fwrite(&t32, 4, 1, lr) == 1;
        if (lr) std::fclose(lr);
        if (!ok) {
            std::fprintf(stderr, "gpat_run: cannot write %slatest_restart\n", restart.c_str());
            gpat_destroy(h);
            return 1;
        }
    }
    gpat_destroy(h);
    return 0;
}
