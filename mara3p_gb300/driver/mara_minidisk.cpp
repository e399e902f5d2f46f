// mara_minidisk — the binary-minidisk driver of problems/minidisk.cpp on the
// GB300 path: host C++17 over the extern "C" layer of libmara_gb300.
//
//   mara_minidisk [key=value ...]
//
// Behaviour follows the reference driver (problems/minidisk.cpp:270-310):
//   - the configuration is the reference's template (problems/minidisk.hpp:99-122)
//     updated by the restart file's run_config, then by the command line;
//     unknown keys are an error;
//   - while time < orbits * 2 pi: checkpoint side effect, then one batch of
//     `fold` steps, then the line "[%06ld] orbit=%lf kzps=%lf" (kzps =
//     1e-3 * fold * cells / seconds, :296-304);
//   - a batch of fold forward-Euler steps uses the dt of the fixed formula at
//     the batch's start (encode_step, :202-213);
//   - checkpoints every `cpi` orbits (side_effects, :239-264) hold git_commit,
//     run_config, schedule {checkpoint, time_series} {next_due, count} and
//     solution {iteration, time, conserved/<level:i-j>} with each block's
//     conserved tuples (n, n, 3). The reference writes them as HDF5 groups;
//     HDF5 is not available here, so the same tree is written as a directory
//     chkpt.%04d/ of JSON files and raw little-endian float64 blocks.
// Extensions (not in the reference): plm_theta (the reference hard-codes 2),
// rk (the reference's driver is forward Euler), precision fp64|mixed,
// dt formula|cfl, seed / perturbation (seeded density perturbation of the
// initial state), graph (replay each fold batch from a CUDA graph), dry
// (print the configuration and exit without touching the GPU), and tsi:
// every tsi orbits the time_series side effect (the schedule entry the
// reference keeps but never writes, problems/minidisk.hpp:64-68; listed as
// to do at problems/minidisk.cpp:69) appends one row to time_series.dat:
// time, iteration, the time integrals of the diagnostics rate vector
// (mara_minidisk_diagnostics, accumulated on the device every step), the
// last step's mean rates, the binary's semi-major axis and eccentricity
// (two_body::recover_orbital_elements) and the rates of (a, M, q, e) that
// the gas's forces and accretion imply. Checkpoints carry the integrals
// (time_series.json), so a restart continues them.
#include <cuda_runtime.h>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <tuple>
#include <cctype>
#include <string>
#include <vector>
#include "mara_gb300.h"

namespace fs = std::filesystem;

namespace {

// ---------------------------------------------------------------- configuration
struct Item
{
    std::string key, kind, value, help;   // kind: int, double, string
};

std::vector<Item> config_template()
{
    return {
        {"block_size", "int", "64", "number of zones per side"},
        {"depth", "int", "1", "number of levels in the mesh"},
        {"omega_frame", "double", "1.0", "reference frame rotation frequency (1.0 for co-rotating)"},
        {"mach_number", "double", "10.0", "Mach number of the disk"},
        {"nu", "double", "0.0", "Kinematic viscosity coefficient"},
        {"domain_radius", "double", "1.5", "half-size of the domain"},
        {"eccentricity", "double", "0.0", "binary orbital eccentricity"},
        {"mass_ratio", "double", "1.0", "binary mass ratio M2 / M1"},
        {"softening_length", "double", "0.01", "gravitational softening length"},
        {"sink_radius", "double", "0.01", "radius of mass sinks"},
        {"sink_rate", "double", "1e3", "rate of mass and momentum removal at sinks"},
        {"buffer_rate", "double", "1e2", "maximum rate of buffer driving"},
        {"buffer_scale", "double", "0.2", "length scale of buffer onset"},
        {"cfl", "double", "0.3", "Courant number"},
        {"orbits", "double", "100.0", "time to stop the simulation"},
        {"cpi", "double", "0.1", "number of orbits between checkpoints"},
        {"threads", "int", "1", "number of threads to execute on (unused: one GPU)"},
        {"fold", "int", "1", "number of encodings per time step batch"},
        {"restart", "string", "", "a checkpoint to restart from"},
        {"outdir", "string", ".", "the directory where output files are written"},
        {"plm_theta", "double", "2.0", "PLM theta (the reference hard-codes 2.0)"},
        {"rk", "int", "1", "Runge-Kutta order, 1 or 2 (the reference driver: 1)"},
        {"precision", "string", "fp64", "fp64 (drop-in) or mixed (FP32 fluxes, FP64 state)"},
        {"dt", "string", "formula", "formula (held over a fold batch) or cfl"},
        {"seed", "int", "0", "seed of the initial density perturbation"},
        {"perturbation", "double", "0.0", "relative amplitude of the initial density perturbation"},
        {"graph", "int", "1", "replay each fold batch from a CUDA graph"},
        {"dry", "int", "0", "print the configuration and exit"},
        {"tsi", "double", "0.0", "number of orbits between time-series samples (0: none)"},
    };
}

class Config
{
public:
    Config() : items_(config_template()) {}

    void update(const std::map<std::string, std::string>& kv)
    {
        for (const auto& [k, v] : kv) set(k, v);
    }

    void set(const std::string& key, const std::string& value)
    {
        for (auto& it : items_)
            if (it.key == key)
            {
                check(it, value);
                it.value = value;
                return;
            }
        throw std::invalid_argument("unknown configuration key '" + key + "'");
    }

    std::string str(const std::string& key) const { return find(key).value; }
    int get_int(const std::string& key) const { return std::stoi(find(key).value); }
    double get_double(const std::string& key) const { return std::stod(find(key).value); }
    const std::vector<Item>& items() const { return items_; }

    // mara::pretty_print layout: header, then key ......... value
    void print(FILE* f) const
    {
        std::fprintf(f, "%s\nconfig:\n\n", std::string(52, '=').c_str());
        for (const auto& it : items_)
        {
            std::string k = it.key + " ";
            while (k.size() < 24) k += '.';
            std::fprintf(f, "\t%s %s\n", k.c_str(), it.value.c_str());
        }
        std::fprintf(f, "%s\n", std::string(52, '=').c_str());
    }

private:
    const Item& find(const std::string& key) const
    {
        for (const auto& it : items_)
            if (it.key == key) return it;
        throw std::invalid_argument("unknown configuration key '" + key + "'");
    }

    static void check(const Item& it, const std::string& v)
    {
        size_t used = 0;
        try
        {
            if (it.kind == "int") (void)std::stoi(v, &used);
            else if (it.kind == "double") (void)std::stod(v, &used);
            else used = v.size();
        }
        catch (const std::exception&)
        {
            used = 0;
        }
        if (used != v.size() || (it.kind != "string" && v.empty()))
            throw std::invalid_argument("configuration key '" + it.key + "' expects " + it.kind + ", got '" + v + "'");
    }

    std::vector<Item> items_;
};

// ---------------------------------------------------------------- minimal JSON
// Objects of numbers, strings and objects: what the checkpoint files hold.
struct Json
{
    enum Kind { NUMBER, STRING, OBJECT } kind = NUMBER;
    double number = 0.0;
    std::string text;
    std::map<std::string, Json> object;

    const Json& at(const std::string& k) const
    {
        auto it = object.find(k);
        if (it == object.end()) throw std::runtime_error("checkpoint: missing key '" + k + "'");
        return it->second;
    }
};

class JsonReader
{
public:
    explicit JsonReader(std::string s) : s_(std::move(s)) {}

    Json parse()
    {
        Json v = value();
        space();
        if (i_ != s_.size()) fail("trailing characters");
        return v;
    }

private:
    [[noreturn]] void fail(const std::string& what) const
    {
        throw std::runtime_error("checkpoint JSON: " + what + " at offset " + std::to_string(i_));
    }
    void space()
    {
        while (i_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[i_]))) ++i_;
    }
    void expect(char c)
    {
        space();
        if (i_ >= s_.size() || s_[i_] != c) fail(std::string("expected '") + c + "'");
        ++i_;
    }
    std::string string_literal()
    {
        expect('"');
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"')
        {
            if (s_[i_] == '\\' && i_ + 1 < s_.size()) ++i_;
            out += s_[i_++];
        }
        if (i_ >= s_.size()) fail("unterminated string");
        ++i_;
        return out;
    }
    Json value()
    {
        space();
        if (i_ >= s_.size()) fail("unexpected end");
        Json v;
        if (s_[i_] == '{')
        {
            ++i_;
            v.kind = Json::OBJECT;
            space();
            if (i_ < s_.size() && s_[i_] == '}') { ++i_; return v; }
            for (;;)
            {
                std::string k = string_literal();
                expect(':');
                v.object[k] = value();
                space();
                if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
                expect('}');
                return v;
            }
        }
        if (s_[i_] == '"')
        {
            v.kind = Json::STRING;
            v.text = string_literal();
            return v;
        }
        size_t used = 0;
        try
        {
            v.number = std::stod(s_.substr(i_), &used);
        }
        catch (const std::exception&)
        {
            fail("bad number");
        }
        i_ += used;
        return v;
    }

    std::string s_;
    size_t i_ = 0;
};

std::string json_escape(const std::string& s)
{
    std::string out;
    for (char c : s)
    {
        if (c == '"' || c == '\\') out += '\\';
        out += c;
    }
    return out;
}

std::string json_number(double x)
{
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.17g", x);
    return buf;
}

std::string read_file(const fs::path& p)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) throw std::runtime_error("cannot read " + p.string());
    std::ostringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

void write_file(const fs::path& p, const std::string& data)
{
    std::ofstream f(p, std::ios::binary);
    if (!f || !f.write(data.data(), std::streamsize(data.size()))) throw std::runtime_error("cannot write " + p.string());
}

// ---------------------------------------------------------------- blocks
// mesh::format_block_index (src/mesh_block_index.hpp:361-375): "level:i-j",
// coordinates zero-padded to 1 + log10(2^level) digits.
std::string block_name(int level, long i, long j)
{
    const int width = int(1 + std::log10(double(1L << level)));
    char buf[64];
    std::snprintf(buf, sizeof buf, "%d:%0*ld-%0*ld", level, width, i, width, j);
    return buf;
}

struct Schedule
{
    double checkpoint_next_due = 0.0, time_series_next_due = 0.0;
    int checkpoint_count = 0, time_series_count = 0;
};

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void mara_check(int status, const char* what)
{
    if (status != MARA_OK) throw std::runtime_error(std::string(what) + ": " + mara_last_error());
}

mara_minidisk_params solver_data(const Config& c)
{
    mara_minidisk_params p{};
    p.block_size = c.get_int("block_size");
    p.depth = c.get_int("depth");
    p.omega_frame = c.get_double("omega_frame");
    p.mach_number = c.get_double("mach_number");
    p.nu = c.get_double("nu");
    p.domain_radius = c.get_double("domain_radius");
    p.softening_length = c.get_double("softening_length");
    p.eccentricity = c.get_double("eccentricity");
    p.mass_ratio = c.get_double("mass_ratio");
    p.sink_radius = c.get_double("sink_radius");
    p.sink_rate = c.get_double("sink_rate");
    p.buffer_rate = c.get_double("buffer_rate");
    p.buffer_scale = c.get_double("buffer_scale");
    p.cfl = c.get_double("cfl");
    p.plm_theta = c.get_double("plm_theta");
    return p;
}

// The solution on the device: SoA [3][N][N] state and the device clock.
struct Run
{
    mara_minidisk_params p{};
    int N = 0, rk = 1, precision = MARA_FP64, dt_mode = MARA_DT_FORMULA_HELD;
    double* u = nullptr;
    mara_minidisk_clock* clock = nullptr;
    void* workspace = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_fold = 0;
    mara_minidisk_diagnostics* diag = nullptr;   // device; with the time series only

    ~Run()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (diag) cudaFree(diag);
        if (u) cudaFree(u);
        if (clock) cudaFree(clock);
        if (workspace) cudaFree(workspace);
        if (stream) cudaStreamDestroy(stream);
    }

    mara_minidisk_clock read_clock() const
    {
        mara_minidisk_clock c;
        cuda_check(cudaMemcpyAsync(&c, clock, sizeof c, cudaMemcpyDeviceToHost, stream), "read clock");
        cuda_check(cudaStreamSynchronize(stream), "read clock");
        return c;
    }

    // one batch of `fold` steps, from a CUDA graph (captured on first use) or directly
    void batch(int fold, bool use_graph)
    {
        if (!use_graph)
        {
            mara_check(mara_minidisk_advance_diag(&p, u, clock, fold, rk, precision, dt_mode, workspace, diag, stream),
                       "advance");
            return;
        }
        if (!graph || graph_fold != fold)
        {
            if (graph) cudaGraphExecDestroy(graph);
            graph = nullptr;
            cudaGraph_t g = nullptr;
            cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed), "begin capture");
            const int r = mara_minidisk_advance_diag(&p, u, clock, fold, rk, precision, dt_mode, workspace, diag, stream);
            const cudaError_t e = cudaStreamEndCapture(stream, &g);
            mara_check(r, "advance (capture)");
            cuda_check(e, "end capture");
            cuda_check(cudaGraphInstantiate(&graph, g, 0), "instantiate graph");
            cuda_check(cudaGraphUpload(graph, stream), "upload graph");
            cudaGraphDestroy(g);
            graph_fold = fold;
        }
        cuda_check(cudaGraphLaunch(graph, stream), "graph launch");
    }

    mara_minidisk_diagnostics read_diagnostics() const
    {
        mara_minidisk_diagnostics d;
        cuda_check(cudaMemcpyAsync(&d, diag, sizeof d, cudaMemcpyDeviceToHost, stream), "read diagnostics");
        cuda_check(cudaStreamSynchronize(stream), "read diagnostics");
        return d;
    }
};

// ---------------------------------------------------------------- checkpoints
void write_checkpoint(const fs::path& dir, const Config& cfg, const Schedule& sch, Run& run)
{
    const int n = run.p.block_size, nb = 1 << run.p.depth, N = run.N;
    const mara_minidisk_clock c = run.read_clock();
    std::vector<double> u(size_t(3) * N * N);
    cuda_check(cudaMemcpy(u.data(), run.u, u.size() * sizeof(double), cudaMemcpyDeviceToHost), "checkpoint copy");

    const fs::path tmp = dir.string() + ".partial";
    fs::remove_all(tmp);
    fs::create_directories(tmp / "solution" / "conserved");
    write_file(tmp / "git_commit", std::string(mara_version()));
    std::string rc = "{\n";
    for (size_t k = 0; k < cfg.items().size(); ++k)
    {
        const Item& it = cfg.items()[k];
        rc += "  \"" + it.key + "\": " + (it.kind == "string" ? "\"" + json_escape(it.value) + "\"" : it.value);
        rc += k + 1 < cfg.items().size() ? ",\n" : "\n";
    }
    write_file(tmp / "run_config.json", rc + "}\n");
    write_file(tmp / "schedule.json",
               "{\n  \"checkpoint\": {\"next_due\": " + json_number(sch.checkpoint_next_due) + ", \"count\": " +
               std::to_string(sch.checkpoint_count) + "},\n  \"time_series\": {\"next_due\": " +
               json_number(sch.time_series_next_due) + ", \"count\": " + std::to_string(sch.time_series_count) + "}\n}\n");
    write_file(tmp / "solution.json", "{\n  \"iteration\": " + std::to_string(c.iteration) + ",\n  \"time\": " +
                                      json_number(c.time) + "\n}\n");
    if (run.diag)
    {
        const mara_minidisk_diagnostics d = run.read_diagnostics();
        // the integrals keyed by their entry number (the reader knows objects, not arrays)
        std::string ts = "{\n  \"steps\": " + std::to_string(d.steps) + ",\n  \"integral\": {";
        for (int k = 0; k < MARA_DIAG_COUNT; ++k)
            ts += "\"" + std::to_string(k) + "\": " + json_number(d.integral[k]) + (k + 1 < MARA_DIAG_COUNT ? ", " : "");
        write_file(tmp / "time_series.json", ts + "}\n}\n");
    }
    // every block's conserved tuples (n, n, 3), the reference's nd::shared_array layout
    std::string block(size_t(n) * n * 3 * sizeof(double), '\0');
    for (long bi = 0; bi < nb; ++bi)
        for (long bj = 0; bj < nb; ++bj)
        {
            double* b = reinterpret_cast<double*>(block.data());
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j)
                    for (int q = 0; q < 3; ++q)
                        b[(size_t(i) * n + j) * 3 + q] = u[size_t(q) * N * N + size_t(bi * n + i) * N + (bj * n + j)];
            write_file(tmp / "solution" / "conserved" / block_name(run.p.depth, bi, bj), block);
        }
    fs::remove_all(dir);
    fs::rename(tmp, dir);
    std::printf("write %s\n", dir.string().c_str());
}

std::map<std::string, std::string> read_run_config(const fs::path& dir)
{
    const Json j = JsonReader(read_file(dir / "run_config.json")).parse();
    std::map<std::string, std::string> out;
    for (const auto& [k, v] : j.object)
    {
        if (k == "restart" || k == "dry") continue;
        out[k] = v.kind == Json::STRING ? v.text : json_number(v.number);
        if (v.kind == Json::NUMBER && v.number == std::floor(v.number) && std::fabs(v.number) < 1e15)
            out[k] = std::to_string((long long)v.number);
    }
    return out;
}

Schedule read_schedule(const fs::path& dir)
{
    const Json j = JsonReader(read_file(dir / "schedule.json")).parse();
    Schedule s;
    s.checkpoint_next_due = j.at("checkpoint").at("next_due").number;
    s.checkpoint_count = int(j.at("checkpoint").at("count").number);
    s.time_series_next_due = j.at("time_series").at("next_due").number;
    s.time_series_count = int(j.at("time_series").at("count").number);
    return s;
}

// the solution of a checkpoint into the device state; returns (iteration, time)
// The diagnostics integrals of a checkpoint (zero if it has none) into run.diag.
void read_time_series(const fs::path& dir, Run& run)
{
    mara_minidisk_diagnostics d;
    std::memset(&d, 0, sizeof d);
    if (fs::exists(dir / "time_series.json"))
    {
        const Json j = JsonReader(read_file(dir / "time_series.json")).parse();
        d.steps = int64_t(j.at("steps").number);
        for (int k = 0; k < MARA_DIAG_COUNT; ++k) d.integral[k] = j.at("integral").at(std::to_string(k)).number;
    }
    cuda_check(cudaMemcpy(run.diag, &d, sizeof d, cudaMemcpyHostToDevice), "restore diagnostics");
}

std::pair<long, double> read_solution(const fs::path& dir, Run& run)
{
    const Json j = JsonReader(read_file(dir / "solution.json")).parse();
    const int n = run.p.block_size, nb = 1 << run.p.depth, N = run.N;
    std::vector<double> u(size_t(3) * N * N);
    for (long bi = 0; bi < nb; ++bi)
        for (long bj = 0; bj < nb; ++bj)
        {
            const fs::path f = dir / "solution" / "conserved" / block_name(run.p.depth, bi, bj);
            const std::string data = read_file(f);
            if (data.size() != size_t(n) * n * 3 * sizeof(double))
                throw std::runtime_error("checkpoint block " + f.string() + " has the wrong size");
            const double* b = reinterpret_cast<const double*>(data.data());
            for (int i = 0; i < n; ++i)
                for (int jj = 0; jj < n; ++jj)
                    for (int q = 0; q < 3; ++q)
                        u[size_t(q) * N * N + size_t(bi * n + i) * N + (bj * n + jj)] = b[(size_t(i) * n + jj) * 3 + q];
        }
    cuda_check(cudaMemcpy(run.u, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice), "restart copy");
    return {long(j.at("iteration").number), j.at("time").number};
}

int main_impl(int argc, const char* argv[])
{
    // mara::argv_to_string_map: every key=value argument
    std::map<std::string, std::string> args;
    for (int k = 1; k < argc; ++k)
    {
        const std::string a = argv[k];
        const auto eq = a.find('=');
        if (eq == std::string::npos) throw std::invalid_argument("arguments are key=value, got '" + a + "'");
        args[a.substr(0, eq)] = a.substr(eq + 1);
    }
    Config cfg;
    if (args.count("restart") && !args.at("restart").empty()) cfg.update(read_run_config(args.at("restart")));
    cfg.update(args);
    cfg.print(stdout);
    const std::string prec = cfg.str("precision"), dtm = cfg.str("dt");
    if (prec != "fp64" && prec != "mixed") throw std::invalid_argument("precision must be fp64 or mixed");
    if (dtm != "formula" && dtm != "cfl") throw std::invalid_argument("dt must be formula or cfl");
    if (cfg.get_int("fold") < 1) throw std::invalid_argument("fold must be at least 1");
    if (cfg.get_int("rk") != 1 && cfg.get_int("rk") != 2) throw std::invalid_argument("rk must be 1 or 2");
    Run run;
    run.p = solver_data(cfg);
    run.rk = cfg.get_int("rk");
    run.precision = prec == "mixed" ? MARA_MIXED : MARA_FP64;
    run.dt_mode = dtm == "cfl" ? MARA_DT_CFL : MARA_DT_FORMULA_HELD;
    {
        double dt0 = 0;
        mara_check(mara_minidisk_dt_formula(&run.p, 0.0, &dt0), "solver data");   // validates the parameters
    }
    if (cfg.get_int("dry")) return 0;

    run.N = run.p.block_size << run.p.depth;
    const size_t NN = size_t(run.N) * run.N;
    cuda_check(cudaStreamCreateWithFlags(&run.stream, cudaStreamNonBlocking), "stream");
    cuda_check(cudaMalloc(&run.u, 3 * NN * sizeof(double)), "state");
    cuda_check(cudaMalloc(&run.clock, sizeof(mara_minidisk_clock)), "clock");
    const int64_t ws = mara_minidisk_workspace_bytes(&run.p, run.rk, run.precision);
    if (ws < 0) mara_check(MARA_ERR_ARGUMENT, "workspace");
    cuda_check(cudaMalloc(&run.workspace, size_t(std::max<int64_t>(ws, 256))), "workspace");
    const double tsi = cfg.get_double("tsi");
    if (tsi < 0.0) throw std::invalid_argument("tsi must not be negative");
    if (tsi > 0.0)
    {
        cuda_check(cudaMalloc(&run.diag, sizeof(mara_minidisk_diagnostics)), "diagnostics");
        mara_check(mara_minidisk_diagnostics_reset(run.diag, run.stream), "diagnostics");
    }

    Schedule schedule;
    const std::string restart = cfg.str("restart");
    long iteration = 0;
    double time = 0.0;
    if (!restart.empty())
    {
        schedule = read_schedule(restart);
        std::tie(iteration, time) = read_solution(restart, run);
        if (run.diag) read_time_series(restart, run);
    }
    else
    {
        mara_check(mara_minidisk_initial_conserved(&run.p, uint64_t(cfg.get_int("seed")), cfg.get_double("perturbation"),
                                                   run.u, run.stream), "initial state");
    }
    mara_check(mara_minidisk_clock_init(&run.p, run.u, time, run.clock, run.stream), "clock init");
    {
        mara_minidisk_clock c = run.read_clock();
        c.iteration = iteration;
        cuda_check(cudaMemcpy(run.clock, &c, sizeof c, cudaMemcpyHostToDevice), "clock iteration");
    }

    const double binary_period = 2.0 * M_PI;
    const double orbits = cfg.get_double("orbits"), cpi = cfg.get_double("cpi");
    const int fold = cfg.get_int("fold");
    const bool use_graph = cfg.get_int("graph") != 0;
    const fs::path outdir = cfg.str("outdir");
    const fs::path ts_file = outdir / "time_series.dat";
    if (run.diag) fs::create_directories(outdir);
    if (run.diag && restart.empty())
    {
        std::ofstream f(ts_file, std::ios::trunc);
        f << "# time iteration integral[0..15] rate[0..15] a e da/dt dM/dt dq/dt de/dt\n"
             "# rate entries: sink mass 1, 2; sink momentum x1 y1 x2 y2; gas force x1 y1 x2 y2; buffer mass;\n"
             "#   disk mass; disk angular momentum; torque 1, 2; power (integrals of disk mass and angular\n"
             "#   momentum hold their values at the start of the last step)\n";
    }
    auto time_series = [&](double t) {
        const mara_minidisk_diagnostics d = run.read_diagnostics();
        const mara_minidisk_clock c = run.read_clock();
        double mean[MARA_DIAG_COUNT];
        for (int k = 0; k < MARA_DIAG_COUNT; ++k)
            mean[k] = run.rk == 2 ? 0.5 * (d.rate[0][k] + d.rate[1][k]) : d.rate[0][k];
        if (d.steps == 0)
            for (double& m : mean) m = 0.0;
        double b[10], el[10], er[4];
        mara_check(mara_minidisk_binary(&run.p, t, b), "binary");
        mara_check(mara_two_body_elements(b, t, el), "orbital elements");
        mara_check(mara_two_body_element_rates(b, t, mean, er), "element rates");
        std::ofstream f(ts_file, std::ios::app);
        if (!f) throw std::runtime_error("cannot append to " + ts_file.string());
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.17g %lld", t, (long long)c.iteration);
        f << buf;
        auto put = [&](double x) { std::snprintf(buf, sizeof buf, " %.17g", x); f << buf; };
        for (double x : d.integral) put(x);
        for (double x : mean) put(x);
        put(el[0]);
        put(el[3]);
        for (double x : er) put(x);
        f << "\n";
    };
    auto side_effects = [&](double t) {
        if (run.diag && t >= schedule.time_series_next_due)
        {
            schedule.time_series_next_due += tsi * binary_period;
            schedule.time_series_count += 1;
            time_series(t);
        }
        if (t >= schedule.checkpoint_next_due)
        {
            char name[32];
            std::snprintf(name, sizeof name, "chkpt.%04d", schedule.checkpoint_count);
            schedule.checkpoint_next_due += cpi * binary_period;
            schedule.checkpoint_count += 1;
            fs::create_directories(outdir);
            write_checkpoint(outdir / name, cfg, schedule, run);
        }
    };
    std::printf("\trun on 1 GB300 (%s, %s dt, RK%d%s)\n\n", prec.c_str(), dtm.c_str(), run.rk,
                use_graph ? ", fold batches replayed from a CUDA graph" : "");
    while (time < orbits * binary_period)
    {
        side_effects(time);
        const auto t0 = std::chrono::high_resolution_clock::now();
        run.batch(fold, use_graph);
        const mara_minidisk_clock c = run.read_clock();   // synchronises the stream
        const auto t1 = std::chrono::high_resolution_clock::now();
        time = c.time;
        const double seconds = std::chrono::duration<double>(t1 - t0).count();
        const double kzps = 1e-3 * fold * double(NN) / seconds;
        std::printf("[%06ld] orbit=%lf kzps=%lf\n", long(c.iteration), time / 2 / M_PI, kzps);
        std::fflush(stdout);
    }
    side_effects(time);
    return 0;
}

} // namespace

int main(int argc, const char* argv[])
{
    try
    {
        return main_impl(argc, argv);
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "mara_minidisk: %s\n", e.what());
        return 1;
    }
}
