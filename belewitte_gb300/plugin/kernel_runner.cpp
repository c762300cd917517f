// kernel-runner: loads the algorithm libraries and runs jobs, with the
// command-line surface of the reference's kernel-runner.cpp:
//
//   kernel-runner list algorithms [-L PATH]
//   kernel-runner list implementations -a NAME [-v] [-L PATH]
//   kernel-runner query algorithm-version -a NAME
//   kernel-runner query device [-d NUM]
//   kernel-runner -a ALGORITHM -k KERNEL [OPTIONS] <graph file(s)>
//   kernel-runner -S      (jobs read from stdin, one per line, first word = tag)
//
// Libraries are found as lib<name>kernel.so in ./.build/kernels/ and every
// -L path (kernel-runner.cpp:98-148); each exports registerCUDA.  For every
// graph it writes <label>.timings (`name:min mean max stddev` ns) and
// <label>.output in -o DIR and prints `commit:label` (kernel-runner.cpp:222-256).
#include <dirent.h>
#include <dlfcn.h>
#include <regex>
#include <sstream>
#include <sys/stat.h>
#include <wordexp.h>
#ifdef __linux__
#include <pthread.h>
#include <sched.h>
#endif

#include <cuda_runtime_api.h>

#include "framework.hpp"

namespace {

std::map<std::string, Algorithm> algorithms;
std::vector<void *> handles;

bool is_dir(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

void load_algorithms(std::vector<std::string> paths, bool debug)
{
    if (is_dir("./.build/kernels/")) paths.insert(paths.begin(), "./.build/kernels/");
    const std::regex re(debug ? "lib(.*)kerneldebug\\.so" : "lib(.*)kernel\\.so");
    std::map<std::string, std::string> libs;
    for (const auto &dir : paths) {
        DIR *d = opendir(dir.c_str());
        if (!d) continue;
        while (dirent *e = readdir(d)) {
            std::smatch m;
            std::string name = e->d_name;
            if (std::regex_match(name, m, re) && !libs.count(m[1]))
                libs[m[1]] = dir + "/" + name;
        }
        closedir(d);
    }
    for (auto &[name, path] : libs) {
        void *h = dlopen(path.c_str(), RTLD_NOW | RTLD_LOCAL);
        if (!h) {
            std::cerr << "dlopen() failed: " << path << "\n" << dlerror() << std::endl;
            continue;
        }
        auto reg = reinterpret_cast<register_algorithm_t *>(dlsym(h, "registerCUDA"));
        if (!reg) {
            std::cerr << "dlsym() failed: registerCUDA in " << path << std::endl;
            dlclose(h);
            continue;
        }
        handles.push_back(h);
        reg(algorithms[name]);
    }
}

Algorithm &get_algorithm(const std::string &name)
{
    auto it = algorithms.find(name);
    if (it == algorithms.end()) {
        std::ostringstream names;
        for (auto &a : algorithms) names << "    " << a.first << "\n";
        reportError((name.empty() ? std::string("Algorithm name not specified!")
                                  : "No algorithm named \"" + name + "\"!") +
                    "\n\nSupported algorithms:\n" + names.str());
    }
    return it->second;
}

std::string stem(const std::string &path)
{
    std::string base = path.substr(path.find_last_of('/') == std::string::npos ? 0 : path.find_last_of('/') + 1);
    auto dot = base.find_last_of('.');
    return dot == std::string::npos ? base : base.substr(0, dot);
}

struct Globals {
    int device = 0;
    std::vector<std::string> libs;
    std::string out_dir = ".";
    bool print_stdout = false, debug = false, verbose = false, warn = false, from_stdin = false, quiet = false;
    std::string algorithm, kernel;
} G;

void run_job(const std::string &algo, const std::string &kern, const std::vector<std::string> &args,
             const std::string &tag = "")
{
    Algorithm &a = get_algorithm(algo);
    a.selectKernel(kern);
    auto graphs = a.setup(args);
    if (!tag.empty() && graphs.size() > 1) reportError("Tagged output with more than 1 graph!");
    for (const auto &graph : graphs) {
        const std::string label = tag.empty() ? stem(graph) : tag;
        std::string timings = G.out_dir + "/" + label + ".timings";
        std::string output = G.out_dir + "/" + label + ".output";
        if (G.quiet) timings = output = "/dev/null";
        {
            Epoch epoch(G.print_stdout ? "/dev/stdout" : timings, G.verbose);
            a(graph, output);
        }
        std::cout << a.commit() << ":" << label << std::endl;
    }
}

void pin_cpu()
{
#ifdef __linux__
    cpu_set_t set;
    CPU_ZERO(&set);
    CPU_SET(0, &set);
    pthread_setaffinity_np(pthread_self(), sizeof set, &set);   // best effort (kernel-runner.cpp:258-279)
#endif
}

std::vector<std::string> split_words(const std::string &line)
{
    std::vector<std::string> out;
    wordexp_t w;
    if (wordexp(line.c_str(), &w, WRDE_NOCMD | WRDE_UNDEF) != 0) reportError("Failed to expand commandline!");
    for (size_t i = 0; i < w.we_wordc; i++) out.push_back(w.we_wordv[i]);
    wordfree(&w);
    return out;
}

}  // namespace

int main(int argc, char **argv)
{
    pin_cpu();
    Options options;
    options.add('d', "device", "NUM", G.device, "Device to use.")
        .add('L', "lib", "PATH", G.libs, "Search path for algorithm libraries.")
        .add('o', "output-dir", "DIR", G.out_dir, "Location to use for writing algorithm output.")
        .add('O', "output", G.print_stdout, true, "Print timings to stdout, inhibits timings file creation.")
        .add('g', "debug", G.debug, true, "Use debug kernels.")
        .add('v', "verbose", G.verbose, true, "Verbose output.")
        .add('W', "warn", G.warn, true, "Verbose/debug warnings.")
        .add('S', "stdin", G.from_stdin, true, "Read work from stdin.")
        .add('q', "quiet", G.quiet, true, "Inhibit creation of output and timing files.");
    Options job;
    job.add('a', "algorithm", "NAME", G.algorithm, "Algorithm to use.")
        .add('k', "kernel", "NAME", G.kernel, "Which algorithm implementation to use.");

    std::vector<std::string> args(argv + 1, argv + argc);
    bool help = false;
    for (auto &a : args)
        if (a == "-h" || a == "--help") help = true;
    args = job.parse(options.parse(args));
    std::vector<std::string> libs = G.libs.empty() ? std::vector<std::string>{"."} : G.libs;
    load_algorithms(libs, G.debug);

    if (help || (args.empty() && !G.from_stdin)) {
        std::cout << "Usage:\n  kernel-runner list algorithms|implementations\n"
                     "  kernel-runner query algorithm-version|device\n"
                     "  kernel-runner -a ALGORITHM -k KERNEL [OPTIONS] <graph file(s)>\n"
                     "  kernel-runner -S\n\nOptions:\n";
        options.usage(std::cout, "    ");
        job.usage(std::cout, "    ");
        if (!G.algorithm.empty() && !G.kernel.empty()) {
            Algorithm &a = get_algorithm(G.algorithm);
            a.selectKernel(G.kernel);
            a.help(std::cout, "    ");
        }
        return EXIT_SUCCESS;
    }
    if (args.size() >= 2 && args[0] == "list") {
        if (args[1] == "algorithms") {
            for (auto &a : algorithms) std::cout << a.first << std::endl;
            return EXIT_SUCCESS;
        }
        if (args[1] == "implementations") {
            Algorithm &a = get_algorithm(G.algorithm);
            for (auto &[name, impl] : a) {
                std::cout << name << std::endl;
                if (G.verbose) impl->help(std::cout, "    ");
            }
            return EXIT_SUCCESS;
        }
    }
    if (args.size() >= 2 && args[0] == "query") {
        if (args[1] == "algorithm-version") {
            std::cout << get_algorithm(G.algorithm).commit() << std::endl;
            return EXIT_SUCCESS;
        }
        if (args[1] == "device") {
            cudaDeviceProp p;
            if (cudaGetDeviceProperties(&p, G.device) != cudaSuccess) reportError("No such device");
            std::cout << "Device " << G.device << ": " << p.name << ", " << p.multiProcessorCount << " SMs, "
                      << (p.totalGlobalMem >> 20) << " MiB" << std::endl;
            return EXIT_SUCCESS;
        }
    }

    set_device(G.device);
    if (cudaSetDevice(G.device) != cudaSuccess) {
        std::cerr << "Backend not initialised: No devices?" << std::endl;
        return EXIT_FAILURE;
    }
    if (G.from_stdin) {
        std::string line;
        while (std::getline(std::cin, line)) {
            auto words = split_words(line);
            if (words.empty()) continue;
            const std::string tag = words[0];
            std::vector<std::string> rest(words.begin() + 1, words.end());
            rest = job.parse(rest);
            run_job(G.algorithm, G.kernel, rest, tag);
            job.reset();
        }
    } else {
        run_job(G.algorithm, G.kernel, args);
    }
    return EXIT_SUCCESS;
}
