// io.hpp -- output tree, raw float64 monitoring files and the run log,
// laid out like the reference (Cuda-CMM/src/ui/cmm-io.cu:23-64 folders,
// :80-103 raw appends, :692-731 Logger; file names cmm-euler2d.cu:928-959).
#pragma once
#include <cstdio>
#include <string>

#include "settings.hpp"

namespace cmm {

// data/<file_name>/{Monitoring_data{,/Mesure,/Debug_globals},Time_data,Particle_data}
bool create_directory_structure(const Settings& s);
std::string run_dir(const Settings& s);          // <workspace>data/<file_name>
bool append_f64(const std::string& path, const double* v, size_t n);
bool write_f64(const std::string& path, const double* v, size_t n);
bool make_dir(const std::string& path);
// whole-file float64 read of exactly n values: 0 ok, 1 cannot open, 2 file too short
int read_f64(const std::string& path, double* v, size_t n);
// regular files in dir whose name contains sub (countFilesWithString, cmm-simulation-host.cu:1227-1253)
int count_files_containing(const std::string& dir, const std::string& sub);
// "%.3g"-like formatting of std::ostringstream with precision 3
std::string to_str3(double v);
std::string format_duration(double sec);

class Logger {
public:
    explicit Logger(const std::string& path = "");
    ~Logger();
    void open(const std::string& path);
    // the reference's log header (cmm-io.cu:692-709): a fresh run truncates the log and
    // writes the run name; a restarted run appends "Continuing simulation"
    void start(const std::string& path, bool restart, const std::string& run_name);
    void push(const std::string& msg);
    bool quiet = false;   // suppress stdout echo (library use)
private:
    FILE* f_ = nullptr;
};

}  // namespace cmm
