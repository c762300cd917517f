// Framework implementation (linked into kernel-runner and exported to the
// plugin libraries).  See framework.hpp for the reference correspondence.
#include <dlfcn.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <sstream>

#include <cuda_runtime_api.h>

#include "framework.hpp"

double prop_ref::dummy = 0.0;

[[noreturn]] void reportError(const std::string &msg)
{
    std::cerr << msg << std::endl;
    std::exit(EXIT_FAILURE);
}

void check_bw(int status, const std::string &what)
{
    if (status != BW_OK) {
        std::string detail = status == BW_ERR_CUDA ? std::string(" [") + bw_last_error() + "]" : "";
        reportError(what + ": " + bw_status_string(status) + detail);
    }
}

// ----------------------------- tuned launches ------------------------------
namespace {

std::string tuned_file()
{
    if (const char *env = std::getenv("BELEWITTE_AUTOTUNE")) return env;
    Dl_info info{};
    if (!dladdr(reinterpret_cast<void *>(&tuned_config), &info) || !info.dli_fname) return "";
    std::string path = info.dli_fname;
    const size_t slash = path.rfind('/');
    return (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) + "/data/autotune.tsv";
}

// shape class fields: floor(log2(max(n, 2))), floor(log2(average degree, at
// least 1)), floor(log2(max(max out-degree / average degree, 1)))
std::array<int, 3> shape_class(const bw_host_graph &g)
{
    const double n = static_cast<double>(g.vertex_count), m = static_cast<double>(g.edge_count);
    const double avg = std::max(m / std::max(n, 1.0), 1.0);
    uint32_t dmax = 0;
    for (uint64_t v = 0; g.fwd_vertices && v < g.vertex_count; v++)
        dmax = std::max(dmax, g.fwd_vertices[v + 1] - g.fwd_vertices[v]);
    return {static_cast<int>(std::floor(std::log2(std::max(n, 2.0)))), static_cast<int>(std::floor(std::log2(avg))),
            static_cast<int>(std::floor(std::log2(std::max(static_cast<double>(dmax) / avg, 1.0))))};
}

}  // namespace

bw_launch_config tuned_config(const std::string &algorithm, const std::string &variant, const bw_host_graph &g)
{
    bw_launch_config best{};
    std::ifstream in(tuned_file());
    if (!in) return best;
    const std::array<int, 3> cls = shape_class(g);
    int best_dist = 3;                      // farther classes keep the default
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream fields(line);
        std::string algo, name, klass;
        uint32_t b = 0, gr = 0, w = 0, c = 0;
        if (!(fields >> algo >> name >> klass >> b >> gr >> w >> c) || algo != algorithm || name != variant) continue;
        int v = 0, d = 0, k = 0;
        if (std::sscanf(klass.c_str(), "v%d-d%d-s%d", &v, &d, &k) != 3) continue;
        const int dist = std::abs(v - cls[0]) + std::abs(d - cls[1]) + std::abs(k - cls[2]);
        if (dist < best_dist) {
            best_dist = dist;
            best = bw_launch_config{b, gr, w, c, 0};
        }
    }
    return best;
}

static int g_device = 0;
void set_device(int device) { g_device = device; }

bw_context *shared_context()
{
    static bw_context *ctx = [] {
        bw_context *c = nullptr;
        check_bw(bw_context_create(g_device, &c), "bw_context_create");
        return c;
    }();
    return ctx;
}

// ------------------------------- Options ----------------------------------
template<typename T>
static T parse_number(const std::string &s, const std::string &opt)
{
    try {
        size_t used = 0;
        long long v = std::stoll(s, &used, 0);
        if (used != s.size() || v < 0) throw std::invalid_argument(s);
        return static_cast<T>(v);
    } catch (const std::exception &) {
        reportError("Invalid value \"" + s + "\" for option " + opt);
    }
}

Options &Options::add(char s, const std::string &l, const std::string &arg, size_t &v, const std::string &h)
{
    size_t def = v;
    opts_.push_back({s, l, arg, h, [&v, l](const std::string &x) { v = parse_number<size_t>(x, l); },
                     [&v, def] { v = def; }, true});
    return *this;
}

Options &Options::add(char s, const std::string &l, const std::string &arg, int &v, const std::string &h)
{
    int def = v;
    opts_.push_back({s, l, arg, h, [&v, l](const std::string &x) { v = parse_number<int>(x, l); },
                     [&v, def] { v = def; }, true});
    return *this;
}

Options &Options::add(char s, const std::string &l, const std::string &arg, unsigned &v, const std::string &h)
{
    unsigned def = v;
    opts_.push_back({s, l, arg, h, [&v, l](const std::string &x) { v = parse_number<unsigned>(x, l); },
                     [&v, def] { v = def; }, true});
    return *this;
}

Options &Options::add(char s, const std::string &l, const std::string &arg, std::string &v, const std::string &h)
{
    std::string def = v;
    opts_.push_back({s, l, arg, h, [&v](const std::string &x) { v = x; }, [&v, def] { v = def; }, true});
    return *this;
}

Options &Options::add(char s, const std::string &l, const std::string &arg, std::vector<std::string> &v,
                      const std::string &h)
{
    std::vector<std::string> def = v;
    opts_.push_back({s, l, arg, h, [&v](const std::string &x) { v.push_back(x); }, [&v, def] { v = def; }, true});
    return *this;
}

Options &Options::add(char s, const std::string &l, bool &v, bool set_to, const std::string &h)
{
    bool def = v;
    opts_.push_back({s, l, "", h, [&v, set_to](const std::string &) { v = set_to; }, [&v, def] { v = def; }, false});
    return *this;
}

Options &Options::add(const std::string &l, bool &v, bool set_to, const std::string &h)
{ return add('\0', l, v, set_to, h); }

const Options::Opt *Options::find(const std::string &t) const
{
    for (const auto &o : opts_) {
        if (t.size() == 2 && t[0] == '-' && o.short_name && t[1] == o.short_name) return &o;
        if (t.size() > 2 && t.rfind("--", 0) == 0 && t.substr(2) == o.long_name) return &o;
    }
    return nullptr;
}

std::vector<std::string> Options::parse(const std::vector<std::string> &args)
{
    std::vector<std::string> rest;
    for (size_t i = 0; i < args.size(); i++) {
        std::string tok = args[i], value;
        bool inline_value = false;
        if (tok.rfind("--", 0) == 0 && tok.find('=') != std::string::npos) {
            value = tok.substr(tok.find('=') + 1);
            tok = tok.substr(0, tok.find('='));
            inline_value = true;
        }
        const Opt *o = find(tok);
        if (!o) { rest.push_back(args[i]); continue; }
        if (o->takes_value) {
            if (!inline_value) {
                if (i + 1 >= args.size()) reportError("Option " + tok + " needs a value");
                value = args[++i];
            }
            o->set(value);
        } else {
            o->set("");
        }
    }
    return rest;
}

std::vector<std::string> Options::parseFinal(const std::vector<std::string> &args)
{
    std::vector<std::string> rest = parse(args);
    for (const auto &r : rest)
        if (r.size() > 1 && r[0] == '-') reportError("Unknown option: " + r);
    return rest;
}

void Options::reset()
{
    for (auto &o : opts_) o.reset();
}

void Options::usage(std::ostream &out, const std::string &prefix) const
{
    for (const auto &o : opts_) {
        out << prefix;
        if (o.short_name) out << "-" << o.short_name << " ";
        out << "--" << o.long_name;
        if (o.takes_value) out << " " << o.arg;
        out << "    " << o.help << "\n";
    }
}

// ------------------------------- Timers -----------------------------------
namespace {
struct TimerEntry {
    std::string name;
    std::shared_ptr<std::vector<double>> timings;
};
std::vector<TimerEntry> &registry()
{
    static std::vector<TimerEntry> r;
    return r;
}
}  // namespace

Timer::Timer(const std::string &name, size_t reserve)
{
    for (auto &e : registry()) {
        if (e.name == name) { timings_ = e.timings; return; }
    }
    timings_ = std::make_shared<std::vector<double>>();
    timings_->reserve(reserve);
    registry().push_back({name, timings_});
}

void Timer::start() { begin_ = std::chrono::steady_clock::now(); }

void Timer::stop()
{
    auto d = std::chrono::steady_clock::now() - begin_;
    timings_->push_back(static_cast<double>(std::chrono::duration_cast<std::chrono::nanoseconds>(d).count()));
}

void Timer::record_ns(double ns) { timings_->push_back(ns); }

Epoch::Epoch(const std::string &file, bool human) : file_(file), human_(human) { registry().clear(); }

Epoch::~Epoch()
{
    std::ofstream out(file_);
    out.imbue(std::locale("C"));
    for (auto &e : registry()) {
        auto &t = *e.timings;
        if (t.empty()) continue;
        // utils/StatisticalSummary.hpp conventions: min, mean, max and the
        // sample standard deviation (Welford), integer nanoseconds.
        double mn = *std::min_element(t.begin(), t.end()), mx = *std::max_element(t.begin(), t.end());
        double M = 0, S = 0, total = 0;
        long k = 1;
        for (double v : t) {
            total += v;
            double old = M;
            M += (v - old) / static_cast<double>(k);
            S += (v - old) * (v - M);
            k++;
        }
        double mean = total / static_cast<double>(t.size());
        double sd = (k - 2 == 0) ? 0.0 : std::sqrt(S / static_cast<double>(k - 2));
        if (human_) {
            out << e.name << " (" << t.size() << "): min " << mn / 1e6 << " ms, avg " << mean / 1e6
                << " ms, max " << mx / 1e6 << " ms, std " << sd / 1e6 << " ms\n";
        } else {
            out << e.name << ":" << static_cast<long long>(mn) << " " << static_cast<long long>(mean) << " "
                << static_cast<long long>(mx) << " " << static_cast<long long>(sd) << "\n";
        }
    }
    registry().clear();
}

// ----------------------------- Implementations ----------------------------
ImplementationBase::ImplementationBase() : run_count(1), validate_(false), validate(validate_)
{
    options.add('n', "count", "NUM", run_count, "Number of times to run algorithm.");
    options.add("validate", validate_, true, "Output validation results.");
}

ImplementationBase::~ImplementationBase() {}

void ImplementationBase::operator()(const std::string &graphFile, const std::string &output)
{
    std::ofstream out(output);
    prepareRun();
    loadGraph(graphFile);
    runImplementation(out);
    freeGraph();
    cleanupRun();
    options.reset();
}

void Algorithm::selectKernel(const std::string &name)
{
    if (commitHash.empty()) reportError("Algorithm version not specified!");
    auto it = implementations.find(name);
    if (it == implementations.end() || !it->second) {
        std::ostringstream names;
        for (auto &k : implementations) names << "    " << k.first << "\n";
        reportError((name.empty() ? std::string("Kernel name not specified!")
                                  : "No kernel named \"" + name + "\" exists!") +
                    "\n\nSupported kernels:\n" + names.str());
    }
    selected = it->second.get();
}

void Algorithm::addImplementation(const std::string &name, std::unique_ptr<ImplementationBase> &&impl)
{
    if (!implementations.emplace(name, std::move(impl)).second)
        reportError("Implementation with name \"" + name + "\" already exists!");
}

void Algorithm::operator()(const std::string &graphFile, const std::string &output)
{
    if (!selected) reportError("No kernel selected to run!");
    (*selected)(graphFile, output);
}

void Algorithm::help(std::ostream &out, const std::string &prefix)
{
    if (!selected) reportError("No kernel selected!");
    selected->help(out, prefix);
}

std::vector<std::string> Algorithm::setup(const std::vector<std::string> &args)
{
    if (!selected) reportError("No kernel selected!");
    return selected->setup(args);
}

// ------------------------------- Graph loading ----------------------------
void LoadedGraph::load(const std::string &file, int reps)
{
    free();
    check_bw(bw_graph_file_read(file.c_str(), &host), "Failed to open graph " + file);
    const uint64_t n = host.vertex_count, m = host.edge_count;
    auto dev = [&](const void *src, size_t bytes) -> uint32_t * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 4) != cudaSuccess) reportError("cudaMalloc failed");
        allocations.push_back(p);
        if (src && bytes && cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
            reportError("cudaMemcpy failed");
        return static_cast<uint32_t *>(p);
    };
    view = bw_graph_view{};
    view.vertex_count = n;
    view.edge_count = m;
    uint32_t *fv = dev(host.fwd_vertices, (n + 1) * 4), *fe = dev(host.fwd_edges, m * 4);
    uint32_t *rv = fv, *re = fe;
    if (!host.undirected) {
        rv = dev(host.rev_vertices, (n + 1) * 4);
        re = dev(host.rev_edges, m * 4);
    }
    view.fwd_vertices = fv; view.fwd_edges = fe; view.rev_vertices = rv; view.rev_edges = re;
    uint32_t *fin = nullptr, *rin = nullptr;
    if (reps & (4 | 16)) {
        fin = dev(nullptr, m * 4);
        check_bw(bw_expand_edge_list(fv, n, m, fin, nullptr), "bw_expand_edge_list");
    }
    if (reps & (8 | 32)) {
        rin = host.undirected && fin ? fin : dev(nullptr, m * 4);
        if (rin != fin) check_bw(bw_expand_edge_list(rv, n, m, rin, nullptr), "bw_expand_edge_list");
    }
    if (reps & 4) view.fwd_in_edges = fin;
    if (reps & 8) view.rev_in_edges = rin;
    if (reps & 16) {
        uint32_t *s = dev(nullptr, m * 8);
        check_bw(bw_build_struct_edges(fin, fe, m, s, nullptr), "bw_build_struct_edges");
        view.fwd_struct_edges = s;
    }
    if (reps & 32) {
        uint32_t *s = dev(nullptr, m * 8);
        check_bw(bw_build_struct_edges(rin, re, m, s, nullptr), "bw_build_struct_edges");
        view.rev_struct_edges = s;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) reportError("graph transfer failed");
}

void LoadedGraph::free()
{
    for (void *p : allocations) cudaFree(p);
    allocations.clear();
    if (host.fwd_vertices) bw_host_graph_free(&host);
    host = bw_host_graph{};
    view = bw_graph_view{};
}
