// anne_gpu.cpp - the reference's `anne` command line over the GPU engine.
//
//     anne-gpu <Mode> <IDO file> <Type> <Record> <UpIact> [--mixed]
//
// Same arguments and outputs as anne (Anne.cpp:24-36, 38-160): Mode `analysis` runs
// SimMediator::Run until t >= t_stop; Type is accepted as anne accepts it (safe, near, nbs,
// leap); the FP64 engine builds the NBS candidate list, or the Leap one for `leap`, with UpIact
// as the rebuild interval (for safe and near, which list more candidate pairs, the contacts are
// the same while the order of the FP64 impulse sums, and so the last bits, are NBS's).
// Every Record steps <IDO>_NNNNNNN.ido is written and terminate.ido at the end
// (Consultant::RecordIDO, NBSConsultant::NextStep).  --mixed runs the mixed-precision form
// instead (UpIact is then ignored: its list is rebuilt by displacement).  Mode `redistribute`
// (quasi-static ReDistribute) is not part of the GPU engine.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/vedo_gpu.h"

static int usage() {
    std::printf("Usage: anne-gpu <Mode> <IDO file> <Type> <Record> <UpIact> [--mixed]\n"
                "Mode                : analysis\n"
                "Type                : (I)  safe/near\n"
                "                      (II) nbs/leap\n"
                "Record              : integer\n"
                "UpIact (for Type II): integer\n");
    return 0;
}

static std::string record_name(const std::string& prefix, unsigned long long k) {
    char num[32];
    std::snprintf(num, sizeof(num), "%llu", 10000001ull + k);
    return prefix + "_" + (k < 11000001ull ? std::string(num + 2) : std::string(num)) + ".ido";
}

int main(int argc, char** argv) {
    if (argc < 5) return usage();
    const std::string mode = argv[1], ido = argv[2], type = argv[3];
    const unsigned record = (unsigned)std::strtoul(argv[4], nullptr, 10);
    unsigned up_iact = 1;
    bool mixed = false;
    for (int k = 5; k < argc; ++k) {
        if (!std::strcmp(argv[k], "--mixed")) mixed = true;
        else if (k == 5) up_iact = (unsigned)std::strtoul(argv[k], nullptr, 10);
    }
    if ((type == "nbs" || type == "leap") && argc < 6) return usage();
    if (type != "safe" && type != "near" && type != "nbs" && type != "leap") return usage();
    if (mode != "analysis") {
        std::fprintf(stderr, "anne-gpu: mode %s is not supported by the GPU engine\n", mode.c_str());
        return 2;
    }
    if (ido.size() < 4 || ido.compare(ido.size() - 4, 4, ".ido") != 0) return usage();
    vedo_engine_opts o;
    vedo_gpu_default_opts(&o);
    o.up_iact = up_iact ? up_iact : 1;
    o.consultant = type == "leap" ? 1u : 0u;
    o.precision = mixed ? VEDO_PRECISION_MIXED : VEDO_PRECISION_FP64;
    o.record = mixed ? 0 : record;           // the mixed form's records are written below
    o.output_prefix = mixed ? nullptr : ido.c_str();
    vedo_gpu_engine* e = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    if (vedo_gpu_create_from_ido(ido.c_str(), &o, &e) != VEDO_OK) {
        std::fprintf(stderr, "anne-gpu: %s\n", vedo_gpu_last_error(nullptr));
        return 1;
    }
    std::printf("%s: %u objects, %llu steps to run (%s form)\n", ido.c_str(), vedo_gpu_num_objects(e),
                (unsigned long long)vedo_gpu_steps_remaining(e), mixed ? "mixed" : "FP64");
    unsigned long long done = 0, records = 0;
    uint64_t left = vedo_gpu_steps_remaining(e);
    while (left > 0) {
        uint64_t k = left < (1u << 20) ? left : (1u << 20);
        if (mixed && record) k = std::min<uint64_t>(k, record - (done % record));
        int keep = 0;
        if (vedo_gpu_run(e, (uint32_t)k, &keep) != VEDO_OK) {
            std::fprintf(stderr, "anne-gpu: %s\n", vedo_gpu_last_error(e));
            vedo_gpu_destroy(e);
            return 1;
        }
        done += k;
        left -= k;
        if (mixed && record && done % record == 0 &&
            vedo_gpu_write_ido(e, record_name(ido, records++).c_str()) != VEDO_OK) {
            std::fprintf(stderr, "anne-gpu: %s\n", vedo_gpu_last_error(e));
            vedo_gpu_destroy(e);
            return 1;
        }
    }
    if (mixed) {
        const size_t slash = ido.find_last_of('/');
        const std::string dir = slash == std::string::npos ? std::string() : ido.substr(0, slash + 1);
        if (vedo_gpu_write_ido(e, (dir + "terminate.ido").c_str()) != VEDO_OK) {
            std::fprintf(stderr, "anne-gpu: %s\n", vedo_gpu_last_error(e));
            vedo_gpu_destroy(e);
            return 1;
        }
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("done: %llu steps, t = %.9g s, %.3f s wall\n", done, vedo_gpu_time(e), secs);
    vedo_gpu_destroy(e);
    return 0;
}
