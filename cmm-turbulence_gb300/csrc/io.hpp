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
// "%.3g"-like formatting of std::ostringstream with precision 3
std::string to_str3(double v);
std::string format_duration(double sec);

class Logger {
public:
    explicit Logger(const std::string& path = "");
    ~Logger();
    void open(const std::string& path);
    void push(const std::string& msg);
    bool quiet = false;   // suppress stdout echo (library use)
private:
    FILE* f_ = nullptr;
};

}  // namespace cmm
