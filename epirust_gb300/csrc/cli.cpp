// cli.cpp -- `epirust-gb300`, the standalone engine binary with the flags of the
// reference's engine-app (engine-app/src/main.rs:60-87):
//   -c/--config FILE  -m/--mode standalone  -i/--id ID  -t/--threads N  -o/--output-dir DIR
// Only the standalone mode exists here; kafka and mpi (multi-region travel) are out of scope.
// --threads is accepted for compatibility; the tick runs on the GPU.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/epi_engine.h"
#include "json.hpp"

static void usage() {
    std::fprintf(stderr,
                 "usage: epirust-gb300 [-c config.json] [-m standalone] [-i id] [-t threads] [-o output_dir] [--seed N]\n");
}

int main(int argc, char** argv) {
    std::string config = "config/default.json", mode = "standalone", out_dir = "/tmp", id = "default_engine";
    unsigned long long seed = 0;
    bool have_seed = false;
    for (int k = 1; k < argc; ++k) {
        std::string a = argv[k];
        auto next = [&](const char* name) -> std::string {
            if (k + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", name); std::exit(2); }
            return argv[++k];
        };
        if (a == "-c" || a == "--config") config = next("--config");
        else if (a == "-m" || a == "--mode") mode = next("--mode");
        else if (a == "-i" || a == "--id") id = next("--id");
        else if (a == "-t" || a == "--threads") (void)next("--threads");
        else if (a == "-o" || a == "--output-dir") out_dir = next("--output-dir");
        else if (a == "--seed") { seed = std::stoull(next("--seed")); have_seed = true; }
        else if (a == "-h" || a == "--help") { usage(); return 0; }
        else { usage(); return 2; }
    }
    for (auto& ch : mode) ch = (char)std::tolower(ch);
    if (mode != "standalone") {
        std::fprintf(stderr, "mode %s is not supported: only the standalone single-engine run is implemented\n", mode.c_str());
        return 2;
    }
    std::ifstream in(config);
    if (!in) { std::fprintf(stderr, "Failed to read config file %s\n", config.c_str()); return 1; }
    std::stringstream ss;
    ss << in.rdbuf();
    epi_params p;
    char msg[512] = {0};
    if (epi_params_from_json(ss.str().c_str(), &p, msg, sizeof msg) != EPI_OK) {
        std::fprintf(stderr, "Failed to read config file: %s\n", msg);
        return 1;
    }
    if (have_seed) p.seed = seed;
    // enable_citizen_state_messages (common/src/config/mod.rs:55): the per-hour citizen states
    // go to <output_dir>/output/citizen_states_0.bin (the reference publishes them to Kafka)
    bool citizen_states = false;
    try {
        const epi::json::Value root = epi::json::parse(ss.str());
        if (const epi::json::Value* v = root.get("enable_citizen_state_messages"))
            citizen_states = v->kind == epi::json::Value::Bool && v->b;
    } catch (const std::exception&) {
    }
    auto t0 = std::chrono::steady_clock::now();
    epi_engine* h = nullptr;
    int rc;
    if (p.population_source == 1) {  // Population::Csv: the rows of its file
        uint32_t n = 0;
        rc = epi_population_read_csv(p.population_file, nullptr, 0, &n);
        std::vector<uint8_t> flags(n);
        if (rc == EPI_OK) rc = epi_population_read_csv(p.population_file, flags.data(), n, &n);
        if (rc == EPI_OK) rc = epi_engine_create_population(&p, flags.data(), n, &h);
    } else {
        rc = epi_engine_create(&p, &h);
    }
    if (rc != EPI_OK) { std::fprintf(stderr, "engine create failed (%d): %s\n", rc, epi_engine_last_error(nullptr)); return 1; }
    if (citizen_states) {
        const std::string dir = out_dir + "/output";
        std::string mk = "mkdir -p '" + dir + "'";
        if (std::system(mk.c_str()) != 0 ||
            epi_engine_state_stream_open(h, (dir + "/citizen_states_0.bin").c_str()) != EPI_OK) {
            std::fprintf(stderr, "citizen-state stream: %s\n", epi_engine_last_error(h));
            epi_engine_destroy(h);
            return 1;
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    std::vector<epi_counts> rows(p.hours ? p.hours : 1);
    uint32_t n_rows = 0;
    rc = epi_engine_run(h, rows.data(), (uint32_t)rows.size(), &n_rows);
    auto t2 = std::chrono::steady_clock::now();
    if (rc == EPI_OK) rc = epi_engine_state_stream_close(h);
    if (rc != EPI_OK) { std::fprintf(stderr, "run failed (%d): %s\n", rc, epi_engine_last_error(h)); epi_engine_destroy(h); return 1; }
    // the standalone engine id is "0" (engine/src/engine_app.rs:30, 100-101)
    rc = epi_engine_write_outputs(h, out_dir.c_str(), "0");
    if (rc != EPI_OK) { std::fprintf(stderr, "output failed: %s\n", epi_engine_last_error(h)); epi_engine_destroy(h); return 1; }
    double init_s = std::chrono::duration<double>(t1 - t0).count();
    double run_s = std::chrono::duration<double>(t2 - t1).count();
    std::printf("Initialization completed in %.3f seconds\n", init_s);
    std::printf("Number of iterations: %u, Total Time taken %.3f seconds\n", n_rows, run_s);
    std::printf("Iterations/sec: %.1f\n", run_s > 0 ? n_rows / run_s : 0.0);
    epi_engine_destroy(h);
    return 0;
}
