#include "NbodySystem.hpp"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>

namespace gb300 {

NbodySystem::NbodySystem(const OptionsParser &op)
    : gpus(op.gpus), iterations(0), n(0), snapshot_number(op.snapshot_number),
      length_snap(op.length_output_number), force_mode(op.force_mode), host_steps(op.host_steps),
      eta(op.eta), total_mass(0.f), integration_time(op.integration_time), interval_time(op.interval_time),
      snapshot_time(op.snapshot_time), resume(op.resume), resume_info(op.resume_info), max_mass(0.f),
      input_filename(op.input_filename), output_filename(op.output_filename), resume_filename(op.resume_filename),
      snapshot_filename(op.snapshot_filename), h_id(nullptr), h_move(nullptr), h_t(nullptr), h_dt(nullptr),
      h_r(nullptr), h_v(nullptr), h_a2(nullptr), h_a3(nullptr), h_f(nullptr), h_old(nullptr) {
    ops = op.ops;
    // NbodySystem.cpp:50: the product of two floats, kept as a float.
    const float e2f = op.softening * op.softening;
    e2 = (double)e2f;
    en.ini = en.end = en.tmp = en.kinetic = en.potential = 0.0;
    gtime = Gtime();
}

NbodySystem::~NbodySystem() { free_base_attributes(); }

bool NbodySystem::read_input_file() {
    total_mass = 0;
    max_mass = 0.0f;
    bool got_time = false;
    // a resumed run reads the snapshot the info file names (NbodySystem.cpp:86-95)
    const std::string &path = resume_info ? snapshot_filename : input_filename;
    std::ifstream file(path.c_str());
    if (!file.is_open()) {
        std::cerr << "gravidy: cannot open " << path << std::endl;
        return false;
    }
    std::string line;
    std::getline(file, line);
    while (file.good()) {
        if (file.eof()) break;
        const size_t first = line.find_first_not_of(' ');
        if (first != std::string::npos && line[first] == '#') {
            if (!got_time) {
                std::string clean;
                for (char c : line)
                    if (c != '#' && c != ':') clean += (char)std::tolower((unsigned char)c);
                std::istringstream ciss(clean);
                std::vector<std::string> tok((std::istream_iterator<std::string>(ciss)),
                                             std::istream_iterator<std::string>());
                for (size_t t = 0; t + 1 < tok.size(); t++) {
                    if (tok[t] == "time") {
                        snapshot_time = std::strtod(tok[t + 1].c_str(), nullptr);
                        got_time = true;
                        break;
                    }
                }
            }
        } else {
            std::istringstream iss(line);
            std::vector<std::string> tok((std::istream_iterator<std::string>(iss)),
                                         std::istream_iterator<std::string>());
            if (tok.size() != 8) {
                std::cerr << "gravidy: wrong line format in " << path
                          << ": only eight numbers per line are allowed" << std::endl;
                break;
            }
            file_data tmp;
            tmp.id = (int)(unsigned int)std::atoi(tok[0].c_str());
            tmp.m = (float)std::strtod(tok[1].c_str(), nullptr);
            for (int k = 0; k < 3; k++) {
                tmp.r[k] = std::strtod(tok[2 + k].c_str(), nullptr);
                tmp.v[k] = std::strtod(tok[5 + k].c_str(), nullptr);
            }
            if (tmp.m > max_mass) max_mass = tmp.m;
            reader.push_back(tmp);
            total_mass += tmp.m;
        }
        std::getline(file, line);
    }
    n = (unsigned int)reader.size();
    if (n == 0) {
        std::cerr << "gravidy: no particles read from " << input_filename << std::endl;
        return false;
    }
    return true;
}

void NbodySystem::alloc_base_attributes(int) {
    free_base_attributes();
    h_id = new unsigned int[n];
    h_r = new double4[n];
    h_v = new double4[n];
    h_move = new unsigned int[n];
    h_t = new double[n];
    h_dt = new double[n];
    h_a2 = new double3[n];
    h_a3 = new double3[n];
    h_f = new Forces[n];
    h_old = new Forces[n];
    std::memset(h_t, 0, sizeof(double) * n);
    std::memset(h_dt, 0, sizeof(double) * n);
    std::memset(h_f, 0, sizeof(Forces) * n);
    std::memset(h_old, 0, sizeof(Forces) * n);
    std::memset(h_a2, 0, sizeof(double3) * n);
    std::memset(h_a3, 0, sizeof(double3) * n);
    std::memset(h_move, 0, sizeof(unsigned int) * n);
}

void NbodySystem::copy_input_data() {
    for (unsigned int i = 0; i < reader.size(); i++) {
        h_id[i] = (unsigned int)reader[i].id;
        h_r[i].w = reader[i].m;
        h_r[i].x = reader[i].r[0];
        h_r[i].y = reader[i].r[1];
        h_r[i].z = reader[i].r[2];
        h_v[i].x = reader[i].v[0];
        h_v[i].y = reader[i].v[1];
        h_v[i].z = reader[i].v[2];
        h_v[i].w = 0.0;
    }
    std::vector<file_data>().swap(reader);
}

void NbodySystem::free_base_attributes() {
    delete[] h_id; delete[] h_r; delete[] h_v; delete[] h_move; delete[] h_t;
    delete[] h_dt; delete[] h_a2; delete[] h_a3; delete[] h_f; delete[] h_old;
    h_id = h_move = nullptr;
    h_t = h_dt = nullptr;
    h_r = h_v = nullptr;
    h_a2 = h_a3 = nullptr;
    h_f = h_old = nullptr;
}

}  // namespace gb300
