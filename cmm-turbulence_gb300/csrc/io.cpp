// io.cpp -- see io.hpp.
#include "io.hpp"

#include <sys/stat.h>

#include <chrono>
#include <ctime>
#include <filesystem>
#include <sstream>

namespace cmm {

std::string run_dir(const Settings& s) { return s.workspace + "data/" + s.file_name; }

bool make_dir(const std::string& path)
{
    struct stat st;
    if (stat(path.c_str(), &st) == 0) return true;
    return mkdir(path.c_str(), 0777) == 0;
}

bool create_directory_structure(const Settings& s)
{
    bool ok = make_dir(s.workspace + "data");
    std::string base = run_dir(s);
    ok = make_dir(base) && ok;
    if (s.restart_time == 0) {
        std::error_code ec;
        std::filesystem::remove_all(base + "/Monitoring_data", ec);
    }
    ok = make_dir(base + "/Monitoring_data") && ok;
    ok = make_dir(base + "/Monitoring_data/Mesure") && ok;
    if (s.verbose >= 4) ok = make_dir(base + "/Monitoring_data/Debug_globals") && ok;
    ok = make_dir(base + "/Time_data") && ok;
    if (!s.save_zoom.empty()) ok = make_dir(base + "/Zoom_data") && ok;
    if (!s.particles_advected.empty() || !s.particles_forwarded.empty()) ok = make_dir(base + "/Particle_data") && ok;
    return ok;
}

bool append_f64(const std::string& path, const double* v, size_t n)
{
    FILE* f = fopen(path.c_str(), "ab");
    if (!f) return false;
    size_t w = fwrite(v, sizeof(double), n, f);
    fclose(f);
    return w == n;
}

bool write_f64(const std::string& path, const double* v, size_t n)
{
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    size_t w = fwrite(v, sizeof(double), n, f);
    fclose(f);
    return w == n;
}

int read_f64(const std::string& path, double* v, size_t n)
{
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return 1;
    size_t r = fread(v, sizeof(double), n, f);
    fclose(f);
    return r == n ? 0 : 2;
}

int count_files_containing(const std::string& dir, const std::string& sub)
{
    std::error_code ec;
    int n = 0;
    for (std::filesystem::directory_iterator it(dir, ec), end; !ec && it != end; it.increment(ec))
        if (it->is_regular_file(ec) && it->path().filename().string().find(sub) != std::string::npos) n++;
    return n;
}

std::string to_str3(double v)
{
    std::ostringstream os;
    os.precision(3);
    os << v;
    return os.str();
}

std::string format_duration(double sec)
{
    int h = (int)(sec / 3600.0);
    int m = (int)((sec - h * 3600.0) / 60.0);
    double s = sec - h * 3600.0 - m * 60.0;
    std::ostringstream os;
    os.precision(3);
    os << h << "h " << m << "m " << s << "s";
    return os.str();
}

Logger::Logger(const std::string& path) { if (!path.empty()) open(path); }
Logger::~Logger() { if (f_) fclose(f_); }

void Logger::open(const std::string& path)
{
    if (f_) fclose(f_);
    f_ = fopen(path.c_str(), "a");
}

void Logger::start(const std::string& path, bool restart, const std::string& run_name)
{
    if (f_) fclose(f_);
    f_ = fopen(path.c_str(), restart ? "a" : "w");
    if (!f_) return;
    if (restart) fputs("\nContinuing simulation\n\n", f_);
    else fprintf(f_, "%s\n", run_name.c_str());
    fflush(f_);
}

void Logger::push(const std::string& msg)
{
    std::time_t now = std::time(nullptr);
    char buf[64];
    std::strftime(buf, sizeof(buf), "%Y-%m-%d.%X", std::localtime(&now));
    std::string line = std::string("[") + buf + "]\t" + msg + "\n";
    if (f_) { fputs(line.c_str(), f_); fflush(f_); }
    if (!quiet) { fputs(line.c_str(), stdout); fflush(stdout); }
}

}  // namespace cmm
