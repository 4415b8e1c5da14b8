// settings.cpp -- see settings.hpp.
#include "settings.hpp"

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <map>
#include <sstream>

namespace cmm {

namespace {
constexpr double kPi = 3.141592653589793238462643383279502884197169399375105820974944592307816406286208998628034825342117067;
constexpr double kTwoPiS = 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136;

// std::stoi / stod without exceptions escaping: invalid text gives `fallback`
int to_int(const std::string& v, int fallback, bool* ok)
{
    try { size_t p; int r = std::stoi(v, &p); return r; } catch (...) { if (ok) *ok = false; return fallback; }
}
double to_dbl(const std::string& v, double fallback, bool* ok)
{
    try { size_t p; double r = std::stod(v, &p); return r; } catch (...) { if (ok) *ok = false; return fallback; }
}
unsigned long long to_ull(const std::string& v, bool* ok)
{
    try { return std::stoull(v); } catch (...) { if (ok) *ok = false; return 0; }
}

// Iterate "k=v" items of a "{k=v,k=v}" or "\"k=v,...\"" record
// (settings.cu:556-579): records not wrapped in braces or quotes are ignored.
void for_each_item(const std::string& rec, const std::function<void(const std::string&, const std::string&)>& fn)
{
    if (rec.size() < 2) return;
    bool braces = rec.front() == '{' && rec.back() == '}';
    bool quotes = rec.front() == '"' && rec.back() == '"';
    if (!braces && !quotes) return;
    std::string body = rec.substr(1, rec.size() - 2);
    size_t pos = 0;
    while (true) {
        size_t comma = body.find(',', pos);
        std::string item = body.substr(pos, comma == std::string::npos ? std::string::npos : comma - pos);
        size_t eq = item.find('=');
        if (eq != std::string::npos) fn(item.substr(0, eq), item.substr(eq + 1));
        if (comma == std::string::npos) break;
        pos = comma + 1;
    }
}

// "{a,b,c}" -> doubles (settings.h:30-52); returns false if not braced
bool parse_array(const std::string& s, double* out, int max_n)
{
    if (s.empty() || (s.front() != '{' && s.front() != '"') || (s.back() != '}' && s.back() != '"')) return false;
    std::stringstream ss(s.substr(1, s.size() - 2));
    double v;
    int n = 0;
    while (n < max_n && ss >> v) {
        out[n++] = v;
        if (ss.peek() == ',') ss.ignore();
    }
    return true;
}

std::string array_str(const double* a, int n)   // default precision (6): settings.h:53-68
{
    std::ostringstream os;
    os << "{";
    for (int i = 0; i < n; ++i) { os << a[i]; if (i < n - 1) os << ","; }
    os << "}";
    return os.str();
}

int time_integration_number(const std::string& v, int* order)
{
    static const std::map<std::string, std::pair<int, int>> table = {
        {"EulerExp", {10, 1}}, {"RK1", {10, 1}}, {"Heun", {21, 2}}, {"RK2", {21, 2}}, {"AB2", {20, 2}},
        {"RK3", {30, 3}}, {"RK4", {40, 4}}, {"RK3Mod", {31, 3}}, {"RK4Mod", {41, 4}}};
    auto it = table.find(v);
    if (it == table.end()) { *order = 0; return -1; }
    *order = it->second.second;
    return it->second.first;
}

int particle_time_integration_number(const std::string& v)
{
    static const std::map<std::string, int> table = {
        {"EulerExp", 10}, {"RK1", 10}, {"Heun", 20}, {"RK2", 20}, {"RK3", 30}, {"RK4", 40},
        {"RK3Mod", 31}, {"RK4Mod", 41}};
    auto it = table.find(v);
    return it == table.end() ? -1 : it->second;
}

int particle_init_number(const std::string& v)
{
    if (v == "uniform") return 0;
    if (v == "normal" || v == "gaussian") return 1;
    if (v == "circular_ring") return 2;
    if (v == "uniform_grid") return 3;
    if (v == "sine_sheets") return 4;
    return -1;
}
}  // namespace

bool bool_from_string(const std::string& v) { return v == "true" || v == "True" || v == "1"; }

std::string to_str_prec(double v, int prec)
{
    std::ostringstream os;
    os.precision(prec);
    os << v;
    return os.str();
}

std::string str_t(double v) { return to_str_prec(v, 16); }

// ---------------------------------------------------------------- records
void SaveComputational::set_all(const std::string& rec)
{
    for_each_item(rec, [this](const std::string& k, const std::string& v) {
        if (k == "is_instant") is_instant = bool_from_string(v);
        else if (k == "time_start") time_start = to_dbl(v, time_start, nullptr);
        else if (k == "time_end") time_end = to_dbl(v, time_end, nullptr);
        else if (k == "time_step") time_step = to_dbl(v, time_step, nullptr);
        else if (k == "var") var = v;
        else if (k == "conv") conv = bool_from_string(v);
    });
}
std::string SaveComputational::str() const
{
    std::ostringstream os;
    os << "{is_instant=" << (is_instant ? 1 : 0) << ",time_start=" << str_t(time_start);
    if (!is_instant) os << ",time_end=" << str_t(time_end) << ",time_step=" << str_t(time_step);
    os << ",var=" << var << ",conv=" << (conv ? 1 : 0) << "}";
    return os.str();
}

void SaveSample::set_all(const std::string& rec)
{
    for_each_item(rec, [this](const std::string& k, const std::string& v) {
        if (k == "is_instant") is_instant = bool_from_string(v);
        else if (k == "time_start") time_start = to_dbl(v, time_start, nullptr);
        else if (k == "time_end") time_end = to_dbl(v, time_end, nullptr);
        else if (k == "time_step") time_step = to_dbl(v, time_step, nullptr);
        else if (k == "var") var = v;
        else if (k == "grid") grid = to_int(v, grid, nullptr);
    });
}
std::string SaveSample::str() const
{
    std::ostringstream os;
    os << "{is_instant=" << (is_instant ? 1 : 0) << ",time_start=" << str_t(time_start);
    if (!is_instant) os << ",time_end=" << str_t(time_end) << ",time_step=" << str_t(time_step);
    os << ",var=" << var << ",grid=" << grid << "}";
    return os.str();
}

void SaveZoom::set_all(const std::string& rec)
{
    for_each_item(rec, [this](const std::string& k, const std::string& v) {
        if (k == "is_instant") is_instant = bool_from_string(v);
        else if (k == "time_start") time_start = to_dbl(v, time_start, nullptr);
        else if (k == "time_end") time_end = to_dbl(v, time_end, nullptr);
        else if (k == "time_step") time_step = to_dbl(v, time_step, nullptr);
        else if (k == "var") var = v;
        else if (k == "grid") grid = to_int(v, grid, nullptr);
        else if (k == "pos_x") pos_x = to_dbl(v, pos_x, nullptr);
        else if (k == "pos_y") pos_y = to_dbl(v, pos_y, nullptr);
        else if (k == "width_x") width_x = to_dbl(v, width_x, nullptr);
        else if (k == "width_y") width_y = to_dbl(v, width_y, nullptr);
        else if (k == "rep") rep = to_int(v, rep, nullptr);
        else if (k == "rep_fac") rep_fac = to_dbl(v, rep_fac, nullptr);
    });
}
std::string SaveZoom::str() const
{
    std::ostringstream os;
    os << "{is_instant=" << (is_instant ? 1 : 0) << ",time_start=" << str_t(time_start);
    if (!is_instant) os << ",time_end=" << str_t(time_end) << ",time_step=" << str_t(time_step);
    os << ",var=" << var << ",grid=" << grid;
    os << ",pos_x=" << str_t(pos_x) << ",pos_y=" << pos_y << ",width_x=" << str_t(width_x)
       << ",width_y=" << str_t(width_y);
    os << ",rep=" << rep << ",rep_fac=" << str_t(rep_fac) << "}";
    return os.str();
}

void ParticlesAdvected::set_all(const std::string& rec)
{
    for_each_item(rec, [this](const std::string& k, const std::string& v) {
        if (k == "num") num = to_int(v, num, nullptr);
        else if (k == "tau") tau = to_dbl(v, tau, nullptr);
        else if (k == "seed") seed = to_ull(v, nullptr);
        else if (k == "time_integration") { time_integration = v; time_integration_num = particle_time_integration_number(v); }
        else if (k == "init_name") { init_name = v; init_num = particle_init_number(v); }
        else if (k == "init_time") init_time = to_dbl(v, init_time, nullptr);
        else if (k == "init_vel") init_vel = bool_from_string(v);
        else if (k == "init_param_1") init_param[0] = to_dbl(v, init_param[0], nullptr);
        else if (k == "init_param_2") init_param[1] = to_dbl(v, init_param[1], nullptr);
        else if (k == "init_param_3") init_param[2] = to_dbl(v, init_param[2], nullptr);
        else if (k == "init_param_4") init_param[3] = to_dbl(v, init_param[3], nullptr);
    });
}
std::string ParticlesAdvected::str() const
{
    std::ostringstream os;
    os << "{num=" << num << ",tau=" << str_t(tau) << ",seed=" << seed;
    os << ",time_integration=" << time_integration << ",init_name=" << init_name << ",init_time=" << str_t(init_time)
       << ",init_vel=" << (init_vel ? 1 : 0);
    os << ",init_param_1=" << str_t(init_param[0]) << ",init_param_2=" << str_t(init_param[1])
       << ",init_param_3=" << str_t(init_param[2]) << ",init_param_4=" << str_t(init_param[3]) << "}";
    return os.str();
}

void ParticlesForwarded::set_all(const std::string& rec)
{
    for_each_item(rec, [this](const std::string& k, const std::string& v) {
        if (k == "num") num = to_int(v, num, nullptr);
        else if (k == "seed") seed = to_ull(v, nullptr);
        else if (k == "init_name") { init_name = v; init_num = particle_init_number(v); }
        else if (k == "init_time") init_time = to_dbl(v, init_time, nullptr);
        else if (k == "init_param_1") init_param[0] = to_dbl(v, init_param[0], nullptr);
        else if (k == "init_param_2") init_param[1] = to_dbl(v, init_param[1], nullptr);
        else if (k == "init_param_3") init_param[2] = to_dbl(v, init_param[2], nullptr);
        else if (k == "init_param_4") init_param[3] = to_dbl(v, init_param[3], nullptr);
    });
}
std::string ParticlesForwarded::str() const
{
    std::ostringstream os;
    os << "{num=" << num << ",seed=" << seed << ",init_name=" << init_name << ",init_time=" << str_t(init_time);
    os << ",init_param_1=" << str_t(init_param[0]) << ",init_param_2=" << str_t(init_param[1])
       << ",init_param_3=" << str_t(init_param[2]) << ",init_param_4=" << str_t(init_param[3]) << "}";
    return os.str();
}

// ---------------------------------------------------------------- presets
Settings::Settings()
{
    workspace = "./";
    set_simulation_type("cmm_euler_2d");
    sim_name = "debug";
    grid_coarse = 512;
    grid_fine = 2048;
    grid_psi = 1024;
    grid_vort = grid_fine;
    initial_condition = "4_nodes";
    set_initial_condition("4_nodes");
    initial_discrete = false;
    initial_discrete_grid = 2048;
    initial_discrete_location =
        "data/final-state-anticythere-1_gaussian_blobs_C1024_F8192_t3.07e+03_T500/Time_data/Time_270/Vorticity_W_4096.data";
    verbose = 3;
    double b[6] = {0, kTwoPiS, 0, kTwoPiS, 0, 0};
    set_domain_bounds(b);
    final_time = 3;
    set_dt_by_steps = true;
    factor_dt_by_grid = 1;
    steps_per_sec = 20;
    const std::string tmax = str_t(kTMax);
    const char* comp[4] = {"{is_instant=1,time_start=0,var=W-U,conv=1}", nullptr, nullptr, nullptr};
    std::string comp1 = "{is_instant=1,time_start=" + tmax + ",var=W-U,conv=1}";
    std::string comp2 = "{is_instant=0,time_start=0,time_end=" + tmax + ",time_step=0.5,var ,conv=1}";
    std::string comp3 = "{is_instant=0,time_start=0,time_end=" + tmax +
                        ",time_step=0.5,var=PartA_01-PartA_02-PartA_03-PartA_04,conv=0}";
    save_computational.assign(4, SaveComputational());
    save_computational[0].set_all(comp[0]);
    save_computational[1].set_all(comp1);
    save_computational[2].set_all(comp2);
    save_computational[3].set_all(comp3);
    incomp_threshold = 1e-5;
    map_epsilon = 1e-3;
    skip_remapping = false;
    mem_RAM_CPU_remaps = 9000;
    save_map_stack = true;
    restart_time = 0;
    restart_location = "data/debug_4_nodes_C512_F2048_t20_T2.1/MapStack";
    lagrange_order = 0;
    set_time_integration("RK3");
    lagrange_override = -1;
    lagrange_init_higher_order = true;
    set_map_update_order("4th");
    molly_stencil = 0;
    freq_cut_psi = (double)(512) / 4.0;   // preset grid_coarse / 4, fixed at preset time
    save_sample.assign(1, SaveSample());
    save_sample[0].set_all("{is_instant=0,time_start=0,time_end=" + tmax + ",time_step=0.5,var=W,grid=1024}");
    set_scalar_name("rectangle");
    scalar_discrete = false;
    scalar_discrete_grid = 2048;
    scalar_discrete_location = "I-am-not-implemented-yet!";
    save_zoom.clear();
    forward_map = false;
    particles_forwarded.clear();
    const std::string pp = ",init_param_1=" + str_t(kPi) + ",init_param_2=" + str_t(kPi) +
                           ",init_param_3=" + str_t(kPi * 2.0) + ",init_param_4=" + str_t(kPi * 2.0) + "}";
    particles_advected.assign(2, ParticlesAdvected());
    particles_advected[0].set_all("{num=100000,tau=0,seed=0,time_integration=RK3,init_name=sine_sheets,init_time=0,init_vel=0" + pp);
    particles_advected[1].set_all("{num=100000,tau=0.1,seed=0,time_integration=RK3,init_name=uniform,init_time=0,init_vel=0" + pp);
    particles_steps = -1;
}

void Settings::set_simulation_type(const std::string& v)
{
    simulation_type = v;
    if (v == "cmm_euler_2d") simulation_type_num = 0;
    else if (v == "cmm_vlasov_poisson_1d") simulation_type_num = 2;
}

bool Settings::set_initial_condition(const std::string& v)
{
    // initial-condition name tables (settings.h:297-332)
    static const char* euler[] = {"4_nodes", "quadropole", "one_vortex", "two_votices", "three_vortices",
                                  "single_shear_layer", "tanh_shear_layer", "turbulence_gaussienne",
                                  "gaussian_blobs", "shielded_vortex", "two_cosine", "vortex_sheets"};
    static const char* vlasov[] = {"landau_damping", "two_stream", "nonlin_landau_damping"};
    initial_condition = v;
    if (simulation_type == "cmm_vlasov_poisson_1d") {
        for (int i = 0; i < 3; ++i) if (v == vlasov[i]) { initial_condition_num = i; return true; }
    } else {
        for (int i = 0; i < 12; ++i) if (v == euler[i]) { initial_condition_num = i; return true; }
    }
    initial_condition = "zero";
    initial_condition_num = -1;
    error = "unknown initial condition: " + v;
    return false;
}

void Settings::set_time_integration(const std::string& v)
{
    // settings.h:386-398: the Lagrange order is raised, never lowered
    time_integration = v;
    int order = 0;
    time_integration_num = time_integration_number(v, &order);
    if (time_integration_num != -1 && lagrange_order < order) lagrange_order = order;
}

void Settings::set_map_update_order(const std::string& v)
{
    map_update_order = v;
    map_update_order_num = v == "2nd" ? 0 : v == "4th" ? 1 : v == "6th" ? 2 : -1;
}

void Settings::set_scalar_name(const std::string& v)
{
    scalar_name = v;
    scalar_num = v == "rectangle" ? 0 : v == "gaussian" ? 1 : v == "circular_ring" ? 2 : -1;
}

bool Settings::set_domain_bounds(const double* b)
{
    for (int i = 0; i < 6; ++i) domain_bounds[i] = b[i];
    double Lx = domain_bounds[1] - domain_bounds[0], Ly = domain_bounds[3] - domain_bounds[2];
    if (!(Lx > 1e-16 && Ly > 1e-16)) { error = "domain bounds are not positive"; return false; }
    return true;
}

int Settings::set_variable(const std::string& line, const std::string& delim)
{
    size_t pos = line.find(delim);
    if (pos == std::string::npos) return kNoList;
    const std::string k = line.substr(0, pos);
    const std::string v = line.substr(pos + delim.size());
    bool ok = true;
    if (k == "workspace") workspace = v;
    else if (k == "simulation_type") set_simulation_type(v);
    else if (k == "sim_name") sim_name = v;
    else if (k == "grid_coarse") grid_coarse = to_int(v, grid_coarse, &ok);
    else if (k == "grid_fine") grid_fine = to_int(v, grid_fine, &ok);
    else if (k == "grid_psi") grid_psi = to_int(v, grid_psi, &ok);
    else if (k == "grid_vort") grid_vort = to_int(v, grid_vort, &ok);
    else if (k == "domain_bounds") { double b[6] = {0, 0, 0, 0, 0, 0}; parse_array(v, b, 6); set_domain_bounds(b); }
    else if (k == "final_time") final_time = to_dbl(v, final_time, &ok);
    else if (k == "factor_dt_by_grid") factor_dt_by_grid = to_dbl(v, factor_dt_by_grid, &ok);
    else if (k == "steps_per_sec") steps_per_sec = to_int(v, steps_per_sec, &ok);
    else if (k == "set_dt_by_steps") set_dt_by_steps = bool_from_string(v);
    else if (k == "save_computational_num") {
        save_computational.assign(std::max(0, to_int(v, 0, &ok)), SaveComputational());
        if (!ok) error = "bad value for " + k;
        return kListComputational;
    }
    else if (k == "mem_RAM_CPU_remaps") mem_RAM_CPU_remaps = to_int(v, mem_RAM_CPU_remaps, &ok);
    else if (k == "save_map_stack") save_map_stack = bool_from_string(v);
    else if (k == "restart_time") restart_time = to_dbl(v, restart_time, &ok);
    else if (k == "restart_location") restart_location = v;
    else if (k == "verbose") verbose = to_int(v, verbose, &ok);
    else if (k == "initial_condition") set_initial_condition(v);
    else if (k == "initial_params") parse_array(v, initial_params, 10);
    else if (k == "initial_discrete") initial_discrete = bool_from_string(v);
    else if (k == "initial_discrete_grid") initial_discrete_grid = to_int(v, initial_discrete_grid, &ok);
    else if (k == "initial_discrete_location") initial_discrete_location = v;
    else if (k == "incomp_threshold") incomp_threshold = to_dbl(v, incomp_threshold, &ok);
    else if (k == "map_epsilon") map_epsilon = to_dbl(v, map_epsilon, &ok);
    else if (k == "time_integration") set_time_integration(v);
    else if (k == "lagrange_override") lagrange_override = to_int(v, lagrange_override, &ok);
    else if (k == "lagrange_init_higher_order") lagrange_init_higher_order = bool_from_string(v);
    else if (k == "map_update_order") set_map_update_order(v);
    else if (k == "molly_stencil") molly_stencil = to_int(v, molly_stencil, &ok);
    else if (k == "freq_cut_psi") freq_cut_psi = to_dbl(v, freq_cut_psi, &ok);
    else if (k == "skip_remapping") skip_remapping = bool_from_string(v);
    else if (k == "save_sample_num") {
        save_sample.assign(std::max(0, to_int(v, 0, &ok)), SaveSample());
        if (!ok) error = "bad value for " + k;
        return kListSample;
    }
    else if (k == "scalar_name") set_scalar_name(v);
    else if (k == "scalar_discrete") scalar_discrete = bool_from_string(v);
    else if (k == "scalar_discrete_grid") scalar_discrete_grid = to_int(v, scalar_discrete_grid, &ok);
    else if (k == "scalar_discrete_location") scalar_discrete_location = v;
    else if (k == "save_zoom_num") {
        save_zoom.assign(std::max(0, to_int(v, 0, &ok)), SaveZoom());
        if (!ok) error = "bad value for " + k;
        return kListZoom;
    }
    else if (k == "forward_map") forward_map = bool_from_string(v);
    else if (k == "particles_forwarded_num") {
        particles_forwarded.assign(std::max(0, to_int(v, 0, &ok)), ParticlesForwarded());
        if (!ok) error = "bad value for " + k;
        return kListForwarded;
    }
    else if (k == "particles_advected_num") {
        particles_advected.assign(std::max(0, to_int(v, 0, &ok)), ParticlesAdvected());
        if (!ok) error = "bad value for " + k;
        return kListAdvected;
    }
    else if (k == "particles_steps") particles_steps = to_int(v, particles_steps, &ok);
    else if (k == "precision") precision = v;
    else if (k == "psi_upsampler") psi_upsampler = v;
    else if (k == "psi_exact_every") psi_exact_every = to_int(v, psi_exact_every, &ok);
    else if (k == "psi_learned_tol") psi_learned_tol = to_dbl(v, psi_learned_tol, &ok);
    if (!ok) error = "bad value for " + k + ": " + v;
    return kNoList;
}

bool Settings::load_param_file(const std::string& path)
{
    // cmm-param.cu:149-229: header line, "param_version<TAB>=<TAB>n", one
    // skipped line, then key lines; counted record lists follow *_num keys.
    std::ifstream f(path);
    if (!f) { error = "unable to read parameter file " + path; return false; }
    const std::string delim = "\t=\t";
    std::string line;
    if (!std::getline(f, line) || line != "CMM Parameter file") { error = "not a CMM parameter file: " + path; return false; }
    if (!std::getline(f, line)) { error = "truncated parameter file"; return false; }
    size_t p = line.find(delim);
    if (p == std::string::npos || line.substr(0, p) != "param_version") { error = "missing param_version"; return false; }
    std::getline(f, line);   // separator line
    auto next_value = [&](std::string& out) {
        std::string l;
        if (!std::getline(f, l)) { out.clear(); return false; }
        size_t q = l.find(delim);
        out = q == std::string::npos ? std::string() : l.substr(q + delim.size());
        return q != std::string::npos;
    };
    while (std::getline(f, line)) {
        int code = set_variable(line, delim);
        std::string rec;
        switch (code) {
            case kListComputational:
                for (auto& r : save_computational) if (next_value(rec)) r.set_all(rec);
                break;
            case kListSample:
                for (auto& r : save_sample) if (next_value(rec)) r.set_all(rec);
                break;
            case kListZoom:
                for (auto& r : save_zoom) if (next_value(rec)) r.set_all(rec);
                break;
            case kListAdvected:
                for (auto& r : particles_advected) if (next_value(rec)) r.set_all(rec);
                break;
            case kListForwarded:
                for (auto& r : particles_forwarded) if (next_value(rec)) r.set_all(rec);
                break;
            default: break;
        }
    }
    return error.empty();
}

std::string Settings::param_text() const
{
    // cmm-param.cu:39-146 (same key order and value formatting)
    std::ostringstream os;
    auto line = [&os](const std::string& k, const std::string& v) { os << k << "\t=\t" << v << "\n"; };
    auto num = [](double v) { return to_str_prec(v, 16); };
    auto b = [](bool v) { return std::string(v ? "1" : "0"); };
    os << "CMM Parameter file\n";
    line("param_version", "3");
    os << "\n";
    line("workspace", workspace);
    line("simulation_type", simulation_type);
    line("sim_name", sim_name);
    line("grid_coarse", std::to_string(grid_coarse));
    line("grid_fine", std::to_string(grid_fine));
    line("grid_psi", std::to_string(grid_psi));
    line("grid_vort", std::to_string(grid_vort));
    line("domain_bounds", array_str(domain_bounds, 6));
    line("final_time", num(final_time));
    line("set_dt_by_steps", b(set_dt_by_steps));
    if (set_dt_by_steps) line("steps_per_sec", std::to_string(steps_per_sec));
    else line("factor_dt_by_grid", num(factor_dt_by_grid));
    line("save_computational_num", std::to_string(save_computational.size()));
    for (auto& r : save_computational) line("save_computational", r.str());
    line("mem_RAM_CPU_remaps", std::to_string(mem_RAM_CPU_remaps));
    line("save_map_stack", b(save_map_stack));
    line("restart_time", num(restart_time));
    if (restart_time != 0) line("restart_location", restart_location);
    line("verbose", std::to_string(verbose));
    line("initial_condition", initial_condition);
    line("initial_params", array_str(initial_params, 10));
    line("initial_discrete", b(initial_discrete));
    if (initial_discrete) {
        line("initial_discrete_grid", std::to_string(initial_discrete_grid));
        line("initial_discrete_location", initial_discrete_location);
    }
    line("incomp_threshold", num(incomp_threshold));
    line("map_epsilon", num(map_epsilon));
    line("time_integration", time_integration);
    line("lagrange_override", std::to_string(lagrange_override));
    line("lagrange_init_higher_order", b(lagrange_init_higher_order));
    line("map_update_order", map_update_order);
    line("molly_stencil", std::to_string(molly_stencil));
    line("freq_cut_psi", num(freq_cut_psi));
    line("skip_remapping", b(skip_remapping));
    line("save_sample_num", std::to_string(save_sample.size()));
    for (auto& r : save_sample) line("save_sample", r.str());
    line("scalar_name", scalar_name);
    line("scalar_discrete", b(scalar_discrete));
    if (scalar_discrete) {
        line("scalar_discrete_grid", std::to_string(scalar_discrete_grid));
        line("scalar_discrete_location", scalar_discrete_location);
    }
    line("save_zoom_num", std::to_string(save_zoom.size()));
    for (auto& r : save_zoom) line("save_zoom", r.str());
    line("forward_map", b(forward_map));
    if (forward_map) {
        line("particles_forwarded_num", std::to_string(particles_forwarded.size()));
        for (auto& r : particles_forwarded) line("particles_forwarded", r.str());
    }
    line("particles_advected_num", std::to_string(particles_advected.size()));
    for (auto& r : particles_advected) line("particles_advected", r.str());
    if (!particles_advected.empty()) line("particles_steps", std::to_string(particles_steps));
    return os.str();
}

bool Settings::save_param_file(const std::string& path) const
{
    std::ofstream f(path);
    if (!f) return false;
    f << param_text();
    return true;
}

bool Settings::apply_cli(int argc, const char* const* argv)
{
    // main2d.cpp:73-89: every param_file=... is loaded first, then all
    // COMMAND=VALUE arguments are applied (record lists cannot follow on the CLI)
    for (int i = 0; i < argc; ++i) {
        std::string a = argv[i] ? argv[i] : "";
        size_t eq = a.find('=');
        if (eq != std::string::npos && a.substr(0, eq) == "param_file")
            if (!load_param_file(a.substr(eq + 1))) return false;
    }
    for (int i = 0; i < argc; ++i) set_variable(argv[i] ? argv[i] : "", "=");
    return error.empty();
}

double Settings::dt() const
{
    if (set_dt_by_steps) return 1.0 / steps_per_sec;
    return 1.0 / std::max(grid_coarse, grid_coarse) / factor_dt_by_grid;
}

int Settings::effective_lagrange_order() const
{
    // cmm-euler2d.cu:66-76
    int lo = lagrange_order;
    for (auto& p : particles_advected) {
        int need = 0;
        switch (p.time_integration_num) {
            case 20: need = 2; break;
            case 30: case 31: need = 3; break;
            case 40: case 41: need = 4; break;
            default: break;
        }
        if (lo < need) lo = need;
    }
    if (lagrange_override != -1) lo = lagrange_override;
    return lo;
}

int Settings::iter_max() const
{
    return (int)(1.05 * std::ceil((final_time - restart_time) / dt()));
}

int Settings::cpu_map_num() const
{
    // cmm-euler2d.cu:366-367: maps that fit in mem_RAM_CPU_remaps MB
    double map_size = 8.0 * (double)grid_coarse * grid_coarse * sizeof(double) / 1e6;
    int n = (int)(double(mem_RAM_CPU_remaps) / map_size);
    if (forward_map) n = (int)(n / 2.0);
    return n;
}

std::string Settings::derived_file_name() const
{
    // cmm-euler2d.cu:81-83 (to_str of a double uses precision 3)
    auto i = [](int v) { return std::to_string(v); };
    std::string name = sim_name + "_" + initial_condition + "_C" + i(grid_coarse) + "_F" + i(grid_fine) + "_t" +
                       i((int)(1.0 / dt())) + "_T" + to_str_prec(final_time, 3);
    return name;
}

}  // namespace cmm
