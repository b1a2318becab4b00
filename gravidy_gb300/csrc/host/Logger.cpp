#include "Logger.hpp"

#include <sys/stat.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <ctime>
#include <iomanip>
#include <iostream>
#include <sstream>

#include "Timer.hpp"

namespace gb300 {

Logger::Logger(NbodySystem *ns_) : ns(ns_) {
    print_screen = ns->ops.print_screen;
    ofname = ns->output_filename;
    // a run resumed from an info file writes that file again (Logger.cpp:39-50)
    ofname_info = ns->resume_info ? ns->resume_filename : ofname + ".info";
}

std::string Logger::get_timestamp() const {
    time_t now = time(0);
    tm ltm;
    localtime_r(&now, &ltm);
    char buf[64];
    std::snprintf(buf, sizeof(buf), "[%04d-%02d-%02d %02d:%02d:%02d]", 1900 + ltm.tm_year, 1 + ltm.tm_mon,
                  ltm.tm_mday, ltm.tm_hour, ltm.tm_min, ltm.tm_sec);
    return buf;
}

void Logger::print_info() {
    // Logger.cpp:219-237: truncates the .log file when it is the target.
    if (!print_screen) {
        std::ofstream f((ofname + ".log").c_str(), std::ios::out);
    }
}

void Logger::add_info(const std::string &key, const std::string &value) {
    std::ofstream info(ofname_info.c_str(), std::ios_base::app);
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << key << std::setw(20) << std::right
         << value << std::endl;
}

static bool path_exists(const std::string &p) {
    struct stat b;
    return stat(p.c_str(), &b) != -1;
}

// Logger.cpp:136-217: an existing info file is kept as <info>.old, or
// <info>.old<k> with the first free k, before the new one is written.
void Logger::write_info() {
    if (path_exists(ofname_info)) {
        const char last = ofname_info.empty() ? ' ' : ofname_info.back();
        std::string newname = ofname_info + ".old";
        int ext = 0;
        while (path_exists(newname)) {
            if (std::isdigit((unsigned char)last)) ext = (last - '0') + 1;
            newname = ofname_info + ".old" + std::to_string(ext);
            ext++;
        }
        if (std::rename(ofname_info.c_str(), newname.c_str()))
            std::cerr << "gravidy: Failed to rename info file from " << ofname_info << " to " << newname << std::endl;
    }
    std::ofstream info(ofname_info.c_str(), std::ios::out);
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "NumberParticles:" << std::setw(20)
         << std::right << ns->n << std::endl;
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "Softening:" << std::setw(20)
         << std::right << std::sqrt(ns->e2) << std::endl;
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "EtaTimestep:" << std::setw(20)
         << std::right << ns->eta << std::endl;
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "IntegrationTime:" << std::setw(20)
         << std::right << ns->integration_time << std::endl;
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "PrintScreen:" << std::setw(20)
         << std::right << print_screen << std::endl;
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "InputFilename:" << std::setw(20)
         << std::right << ns->input_filename << std::endl;
    info << std::setw(2) << std::left << "#" << std::setw(20) << std::left << "OutputFilename:" << std::setw(20)
         << std::left << ns->output_filename << std::endl;
}

void Logger::write_snapshot(unsigned int snapshot_number, double ITIME) {
    std::ostringstream s;
    s << std::setw(ns->length_snap) << std::setfill('0') << snapshot_number;
    std::ofstream out((ofname + ".snapshot_" + s.str()).c_str(), std::ios::out);
    out << std::fixed;
    out.precision(4);
    out << "# Time:" << std::setw(6) << ITIME << std::endl;
    for (unsigned int i = 0; i < ns->n; i++) {
        out << std::setw(6) << std::right << ns->h_id[i];
        out << std::scientific;
        out << std::setw(15) << std::right << ns->h_r[i].w;
        out << std::setw(15) << std::right << ns->h_r[i].x << std::setw(15) << std::right << ns->h_r[i].y
            << std::setw(15) << std::right << ns->h_r[i].z;
        out << std::setw(15) << std::right << ns->h_v[i].x << std::setw(15) << std::right << ns->h_v[i].y
            << std::setw(15) << std::right << ns->h_v[i].z;
        out << std::endl;
    }
}

void Logger::print_all(double ITIME, unsigned int snapshot_number) {
    std::ofstream file;
    std::ostream *g = &std::cout;
    if (!print_screen) {
        std::ostringstream s;
        s << std::setw(4) << std::setfill('0') << snapshot_number;
        file.open((ofname + ".all.snap_" + s.str()).c_str(), std::ios::out);
        g = &file;
    }
    for (unsigned int i = 0; i < ns->n; i++) {
        *g << std::fixed;
        g->precision(4);
        *g << std::setw(6) << ITIME;
        g->precision(2);
        *g << std::setw(6) << i;
        *g << std::scientific;
        g->precision(6);
        *g << std::setw(15) << std::right << ns->h_r[i].w << std::setw(15) << ns->h_r[i].x << std::setw(15)
           << ns->h_r[i].y << std::setw(15) << ns->h_r[i].z << std::setw(15) << ns->h_v[i].x << std::setw(15)
           << ns->h_v[i].y << std::setw(15) << ns->h_v[i].z;
        for (int c = 0; c < 3; c++) *g << std::setw(15) << ns->h_f[i].a[c];
        for (int c = 0; c < 3; c++) *g << std::setw(15) << ns->h_f[i].a1[c];
        *g << std::setw(15) << ns->h_dt[i] << std::endl;
    }
}

void Logger::print_energy_log(double ITIME, unsigned int iterations, long long interactions, unsigned int nsteps,
                              double new_energy) {
    ns->en.end = new_energy;
    const double rel_error = std::abs((ns->en.end - ns->en.tmp) / ns->en.tmp);
    const double cum_error = std::abs((ns->en.end - ns->en.ini) / ns->en.ini);
    ns->en.tmp = ns->en.end;
    const float time = (float)(wall_seconds() - ns->gtime.integration_ini);
    if (ITIME != 0.0 && ns->gtime.update_end > 0.0)
        ns->gtime.gflops = KERNEL_GFLOP * ((double)interactions / ns->gtime.update_end);

    std::ofstream file;
    std::ostream *g = &std::cout;
    if (!print_screen) {
        file.open((ofname + ".log").c_str(), std::ios::out | std::ios::app);
        g = &file;
    }
    if (ITIME == 0.0) {
        *g << std::setw(2) << std::left << "#" << std::setw(10) << std::right << "IteTime" << std::setw(15)
           << std::right << "Iter" << std::setw(15) << std::right << "Nsteps" << std::setw(20) << std::right
           << "Energy" << std::setw(15) << std::right << "RelE" << std::setw(15) << std::right << "CumE"
           << std::setw(16) << std::right << "ElapsedTime" << std::setw(12) << std::right << "GFLOPS" << std::endl;
    }
    *g << std::fixed << std::setw(2) << std::right << "00";
    g->precision(3);
    *g << std::setw(10) << std::right << ITIME << std::setw(15) << std::right << iterations << std::setw(15)
       << std::right << nsteps;
    *g << std::scientific;
    g->precision(10);
    *g << std::setw(20) << std::right << ns->en.end;
    g->precision(6);
    *g << std::setw(15) << std::right << rel_error << std::setw(15) << std::right << cum_error << std::setw(16)
       << std::right << time;
    *g << std::fixed;
    g->precision(3);
    *g << std::setw(12) << std::right << ns->gtime.gflops << std::endl;
}

void Logger::print_lagrange_radii(double ITIME, const std::vector<double> &radii) {
    std::ofstream file;
    std::ostream *g = &std::cout;
    if (!print_screen) {
        file.open((ofname + ".radii").c_str(), std::ios::out | std::ios::app);
        g = &file;
    }
    *g << "01 " << std::fixed << ITIME << " ";
    g->precision(6);
    for (size_t i = 0; i < radii.size(); i++) *g << std::setw(6) << std::right << radii[i] << " ";
    *g << std::endl;
}

void Logger::log(int type, const std::string &msg) {
    static const char *names[] = {" [ERROR] ", " [WARNING] ", " [SUCCESS] ", " [INFO] "};
    static const char *colors[] = {"\033[0;31m", "\033[0;33m", "\033[0;32m", "\033[0;36m"};
    std::cerr << "\033[0;34m" << get_timestamp() << colors[type] << names[type] << "\033[m" << msg << std::endl;
}

void Logger::log_error(const std::string &msg) { log(0, msg); }
void Logger::log_warning(const std::string &msg) { log(1, msg); }
void Logger::log_success(const std::string &msg) { log(2, msg); }
void Logger::log_info(const std::string &msg) { log(3, msg); }

}  // namespace gb300
