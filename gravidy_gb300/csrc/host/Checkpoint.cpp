#include "Checkpoint.hpp"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>

namespace gb300 {

namespace {
const char MAGIC[8] = {'H', '4', 'C', 'H', 'K', '0', '0', '1'};
}

bool write_checkpoint(const std::string &path, const NbodySystem &ns, const CheckpointScalars &sc) {
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) {
        std::cerr << "gravidy: cannot write checkpoint " << path << std::endl;
        return false;
    }
    const uint64_t n = ns.n;
    bool ok = std::fwrite(MAGIC, 1, 8, fp) == 8;
    ok = ok && std::fwrite(&n, 8, 1, fp) == 1;
    ok = ok && std::fwrite(&sc, sizeof(double), 14, fp) == 14;
    ok = ok && std::fwrite(ns.h_r, sizeof(double4), n, fp) == n;
    ok = ok && std::fwrite(ns.h_v, sizeof(double4), n, fp) == n;
    ok = ok && std::fwrite(ns.h_f, sizeof(Forces), n, fp) == n;
    ok = ok && std::fwrite(ns.h_t, sizeof(double), n, fp) == n;
    ok = ok && std::fwrite(ns.h_dt, sizeof(double), n, fp) == n;
    ok = ok && std::fwrite(ns.h_id, sizeof(unsigned int), n, fp) == n;
    std::fclose(fp);
    if (!ok) std::cerr << "gravidy: short write to " << path << std::endl;
    return ok;
}

bool read_checkpoint(const std::string &path, NbodySystem &ns, CheckpointScalars &sc) {
    FILE *fp = std::fopen(path.c_str(), "rb");
    if (!fp) {
        std::cerr << "gravidy: cannot open checkpoint " << path << std::endl;
        return false;
    }
    char magic[8];
    uint64_t n = 0;
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, MAGIC, 8) == 0;
    ok = ok && std::fread(&n, 8, 1, fp) == 1 && n >= 1 && n < (1ull << 31);
    ok = ok && std::fread(&sc, sizeof(double), 14, fp) == 14;
    if (ok) {
        ns.n = (unsigned int)n;
        ns.alloc_base_attributes(0);
        ok = std::fread(ns.h_r, sizeof(double4), n, fp) == n;
        ok = ok && std::fread(ns.h_v, sizeof(double4), n, fp) == n;
        ok = ok && std::fread(ns.h_f, sizeof(Forces), n, fp) == n;
        ok = ok && std::fread(ns.h_t, sizeof(double), n, fp) == n;
        ok = ok && std::fread(ns.h_dt, sizeof(double), n, fp) == n;
        ok = ok && std::fread(ns.h_id, sizeof(unsigned int), n, fp) == n;
    }
    std::fclose(fp);
    if (!ok) {
        std::cerr << "gravidy: " << path << " is not a complete checkpoint" << std::endl;
        return false;
    }
    ns.e2 = sc.e2;
    ns.eta = (float)sc.eta;
    ns.total_mass = 0.f;   // as read_input_file sums it: float, in particle order
    for (uint64_t i = 0; i < n; i++) ns.total_mass += (float)ns.h_r[i].w;
    ns.iterations = (long long)sc.iterations;
    return true;
}

}  // namespace gb300
