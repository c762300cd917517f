// Plugin framework of the kernel-runner boundary, re-implemented for the
// GB300 libraries.  Same surface as the reference:
//
//   Algorithm            Algorithm.hpp:10-58 (commit stamp, implementation
//                        registry, selectKernel, setup, operator())
//   ImplementationBase   ImplementationBase.hpp:6-33, lifecycle
//                        prepareRun -> loadGraph -> runImplementation ->
//                        freeGraph -> cleanupRun -> options.reset()
//                        (ImplementationBase.cpp:9-19)
//   Options              options/Options.hpp (getopt-style, resettable for
//                        the stdin job mode)
//   Timer / Epoch        Timer.hpp:53-114, output `name:min mean max stddev`
//                        in nanoseconds (Timer.cpp:286-291)
//   prop_ref             ImplementationTemplate.hpp:509-546 (properties the
//                        switch predictor reads by reference)
//   registerCUDA         extern "C" void registerCUDA(Algorithm&), the one
//                        symbol kernel-runner dlsyms (utils/Util.hpp:24)
//
// The framework code (framework_core.cpp) is linked into kernel-runner,
// which exports it (-rdynamic); the plugin libraries resolve against it so
// timers and the registry are shared, as in the reference build.
#pragma once

#include <chrono>
#include <cstdint>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "belewitte_gb300.h"

#ifndef KERNEL_COMMIT
#define KERNEL_COMMIT "belewitte-gb300"
#endif

[[noreturn]] void reportError(const std::string &msg);

// ---------------------------------------------------------------------------
// Options: short (-x VALUE) and long (--name VALUE) options and flags with
// default reset (options/Options.hpp:11-187).
// ---------------------------------------------------------------------------
class Options {
  public:
    Options &add(char s, const std::string &l, const std::string &arg, size_t &v, const std::string &help);
    Options &add(char s, const std::string &l, const std::string &arg, int &v, const std::string &help);
    Options &add(char s, const std::string &l, const std::string &arg, unsigned &v, const std::string &help);
    Options &add(char s, const std::string &l, const std::string &arg, std::string &v, const std::string &help);
    Options &add(char s, const std::string &l, const std::string &arg, std::vector<std::string> &v,
                 const std::string &help);
    Options &add(char s, const std::string &l, bool &v, bool set_to, const std::string &help);
    Options &add(const std::string &l, bool &v, bool set_to, const std::string &help);

    // Parse what this parser knows; unknown arguments are returned.
    std::vector<std::string> parse(const std::vector<std::string> &args);
    // Like parse() but unknown '-' options are an error (final parser).
    std::vector<std::string> parseFinal(const std::vector<std::string> &args);
    void reset();
    void usage(std::ostream &out, const std::string &prefix) const;

  private:
    struct Opt {
        char short_name;
        std::string long_name, arg, help;
        std::function<void(const std::string &)> set;
        std::function<void()> reset;
        bool takes_value;
    };
    std::vector<Opt> opts_;
    const Opt *find(const std::string &token) const;
};

// ---------------------------------------------------------------------------
// Timers
// ---------------------------------------------------------------------------
class Timer {
  public:
    explicit Timer(const std::string &name, size_t reserve = 10);
    void start();
    void stop();
    void record_ns(double ns);         // a device-measured duration

  private:
    std::chrono::steady_clock::time_point begin_;
    std::shared_ptr<std::vector<double>> timings_;
};

// Collects every Timer created while it is alive and prints
// `name:min mean max stddev` (ns) on destruction.
class Epoch {
  public:
    explicit Epoch(const std::string &file, bool human_readable = false);
    ~Epoch();
    Epoch(const Epoch &) = delete;

  private:
    std::string file_;
    bool human_;
};

// ---------------------------------------------------------------------------
// Implementation registry
// ---------------------------------------------------------------------------
struct ImplementationBase {
  protected:
    ImplementationBase();
    Options options;
    size_t run_count;
    bool validate_;

    virtual void loadGraph(const std::string &file) = 0;
    virtual void prepareRun() {}
    virtual void runImplementation(std::ofstream &out) = 0;
    virtual void cleanupRun() {}
    virtual void freeGraph() = 0;

  public:
    ImplementationBase(const ImplementationBase &) = delete;
    void operator=(const ImplementationBase &) = delete;
    virtual ~ImplementationBase();

    const bool &validate;
    void operator()(const std::string &graphFile, const std::string &output);
    void help(std::ostream &out, const std::string &prefix) { options.usage(out, prefix); }
    std::vector<std::string> setup(const std::vector<std::string> &args) { return options.parseFinal(args); }
};

class Algorithm {
  public:
    Algorithm() = default;
    explicit Algorithm(const std::string &commit) : commitHash(commit) {}
    Algorithm(Algorithm &&) = default;
    Algorithm &operator=(Algorithm &&) = default;

    void selectKernel(const std::string &name);
    void addImplementation(const std::string &name, std::unique_ptr<ImplementationBase> &&impl);
    void operator()(const std::string &graphFile, const std::string &output);
    void help(std::ostream &out, const std::string &prefix);
    std::vector<std::string> setup(const std::vector<std::string> &args);
    std::string commit() const { return commitHash; }

    auto begin() { return implementations.begin(); }
    auto end() { return implementations.end(); }

  private:
    std::string commitHash;
    ImplementationBase *selected = nullptr;
    std::map<std::string, std::unique_ptr<ImplementationBase>> implementations;
};

#define INITIALISE_ALGORITHM(x) x = Algorithm(KERNEL_COMMIT)
typedef void register_algorithm_t(Algorithm &);

// ---------------------------------------------------------------------------
// Properties read by a switch predictor (ImplementationTemplate.hpp:509-546):
// a reference to a double that can be re-pointed at the predictor's own
// storage.
// ---------------------------------------------------------------------------
class prop_ref : public std::reference_wrapper<double> {
  public:
    static double dummy;
    prop_ref() : std::reference_wrapper<double>(dummy) {}
    prop_ref(const prop_ref &) = delete;
    prop_ref &operator=(const std::reference_wrapper<double> &v)
    { std::reference_wrapper<double>::operator=(v); return *this; }
    double &operator=(double v) { return this->get() = v; }
    void reset() { std::reference_wrapper<double>::operator=(std::ref(dummy)); }
};

// Device graph loaded from a .graph file in every representation the
// variants read (GraphLoader.hpp:123-211), owned for one run.
struct LoadedGraph {
    bw_host_graph host{};
    bw_graph_view view{};
    std::vector<void *> allocations;
    void load(const std::string &file, int reps);
    void free();
    ~LoadedGraph() { free(); }
};

// The autotuner's launch configuration for `variant` of `algorithm` ("bfs"
// or "pagerank") on graph `g`: the entry for the graph's shape class (log2
// of the vertex count, of the average degree and of the out-degree skew) in
// data/autotune.tsv beside this framework's module, or of the nearest class
// at most two steps away; all zero (the library default) when there is
// none.  The environment variable BELEWITTE_AUTOTUNE names another file.
bw_launch_config tuned_config(const std::string &algorithm, const std::string &variant, const bw_host_graph &g);

void check_bw(int status, const std::string &what);
bw_context *shared_context();   // one context per process (device chosen by kernel-runner)
void set_device(int device);
