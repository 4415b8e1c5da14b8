// settings.hpp -- run settings of the CMM simulation: presets, COMMAND=VALUE
// overrides, {k=v,...} records and the "CMM Parameter file" format.
//
// Drop-in for SettingsCMM (Cuda-CMM/src/ui/settings.h:154-480, settings.cu:
// 18-436) and the param-file reader/writer (src/ui/cmm-param.cu:25-229):
// same keys, same presets, same string tables (initial-condition names,
// time-integration names, map-update orders) and the same precedence
// (presets < param file < command line).  Parsing errors never exit the
// process; they are returned as status codes.
#pragma once
#include <string>
#include <vector>

namespace cmm {

constexpr double kTMax = 10000.0;   // "final" save instant marker (settings.h:26)

struct SaveComputational {
    bool is_instant = false;
    double time_start = 0, time_end = 0, time_step = 0;
    std::string var;
    bool conv = false;
    void set_all(const std::string& rec);
    std::string str() const;
};

struct SaveSample {
    bool is_instant = false;
    double time_start = 0, time_end = 0, time_step = 0;
    std::string var;
    int grid = 0;
    void set_all(const std::string& rec);
    std::string str() const;
};

struct SaveZoom {
    bool is_instant = false;
    double time_start = 0, time_end = 0, time_step = 0;
    std::string var;
    int grid = 0;
    double pos_x = 0, pos_y = 0, width_x = 0, width_y = 0;
    int rep = 0;
    double rep_fac = 0;
    void set_all(const std::string& rec);
    std::string str() const;
};

struct ParticlesAdvected {
    int num = 0;
    double tau = 0;
    unsigned long long seed = 0;
    std::string time_integration;
    int time_integration_num = 0;
    std::string init_name;
    int init_num = 0;
    bool init_vel = false;
    double init_time = 0;
    double init_param[4] = {0, 0, 0, 0};
    void set_all(const std::string& rec);
    std::string str() const;
};

struct ParticlesForwarded {
    int num = 0;
    unsigned long long seed = 0;
    std::string init_name;
    int init_num = 0;
    double init_time = 0;
    double init_param[4] = {0, 0, 0, 0};
    void set_all(const std::string& rec);
    std::string str() const;
};

// Result codes of Settings::set_variable: which record list follows.
enum RecordList { kNoList = 0, kListComputational = 1, kListSample = 2, kListZoom = 3,
                  kListAdvected = 4, kListForwarded = 5 };

class Settings {
public:
    Settings();  // presets (settings.cu:18-327)

    // main
    std::string workspace, simulation_type, sim_name, file_name;
    int simulation_type_num = 0;
    int grid_coarse = 0, grid_fine = 0, grid_psi = 0, grid_vort = 0;
    double domain_bounds[6] = {0, 0, 0, 0, 0, 0};
    double final_time = 0, factor_dt_by_grid = 0;
    int steps_per_sec = 0;
    bool set_dt_by_steps = true;
    std::vector<SaveComputational> save_computational;
    // initial condition
    std::string initial_condition;
    int initial_condition_num = 0;
    double initial_params[10] = {0};
    bool initial_discrete = false;
    int initial_discrete_grid = 0;
    std::string initial_discrete_location;
    int verbose = 0;
    // memory / restart
    int mem_RAM_CPU_remaps = 0;
    bool save_map_stack = false;
    double restart_time = 0;
    std::string restart_location;
    // method
    double incomp_threshold = 0, map_epsilon = 0;
    std::string time_integration;
    int time_integration_num = 0;
    int lagrange_order = 0, lagrange_override = -1;
    bool lagrange_init_higher_order = true;
    std::string map_update_order;
    int map_update_order_num = 0;
    int molly_stencil = 0;
    double freq_cut_psi = 0;
    bool skip_remapping = false;
    std::vector<SaveSample> save_sample;
    // passive scalar
    std::string scalar_name, scalar_discrete_location;
    int scalar_num = 0, scalar_discrete_grid = 0;
    bool scalar_discrete = false;
    std::vector<SaveZoom> save_zoom;
    bool forward_map = false;
    std::vector<ParticlesForwarded> particles_forwarded;
    std::vector<ParticlesAdvected> particles_advected;
    int particles_steps = -1;
    // precision of the map / stream-function arithmetic: "fp64" (reference
    // method) or "mixed" (FP32 displacement maps); not a reference key
    std::string precision = "fp64";
    // learned psi (precision=mixed): upsampler file, exact evaluation every n steps, and the
    // relative L-infinity psi difference above which the exact evaluation takes over; not
    // reference keys
    std::string psi_upsampler;
    int psi_exact_every = 8;
    double psi_learned_tol = 1e-4;

    // status of the last failed parse / validation (empty when fine)
    std::string error;

    void set_time_integration(const std::string& v);
    void set_simulation_type(const std::string& v);
    bool set_initial_condition(const std::string& v);
    void set_map_update_order(const std::string& v);
    void set_scalar_name(const std::string& v);
    bool set_domain_bounds(const double* b);

    // one "command<delim>value" line; returns a RecordList code
    int set_variable(const std::string& line, const std::string& delim);
    // presets < param file(s) named by param_file=... < remaining CLI commands
    bool apply_cli(int argc, const char* const* argv);
    bool load_param_file(const std::string& path);
    bool save_param_file(const std::string& path) const;
    std::string param_text() const;

    // quantities derived in the reference driver (cmm-euler2d.cu:62-83)
    double dt() const;
    int effective_lagrange_order() const;
    int iter_max() const;
    int cpu_map_num() const;
    std::string derived_file_name() const;
};

bool bool_from_string(const std::string& v);
std::string to_str_prec(double v, int prec);   // ostringstream with precision
std::string str_t(double v);                    // precision 16 (settings.h:484-490)

}  // namespace cmm
