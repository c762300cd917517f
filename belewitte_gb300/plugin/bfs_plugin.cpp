// libbfskernel.so: the BFS algorithm library kernel-runner loads.
// Registers every reference BFS implementation name
// (bfs/bfs.cpp:121-223) plus the GB300 variants and `switch`; each runs
// through the C ABI of libbelewitte_gb300.so.
//
// Run semantics follow BFS::runImplementation (bfs/bfs.cpp:51-118): no
// output when the root is out of range; `computation` and per-level
// `N:bfsLevel` timers (device-measured), `resultTransfer`, `graphTransfer`;
// output `vertex \t depth` per vertex, INT_MAX for unreached vertices.
#include <climits>
#include <cuda_runtime_api.h>

#include "framework.hpp"
#include "switching.hpp"

namespace {

struct BfsRun {
    unsigned root = 0;
    size_t warp = 0, chunk = 0;        // -w / -c; 0: tuned, else the library's 32 / 32
    LoadedGraph graph;
    int32_t *levels = nullptr;

    void alloc(uint64_t n)
    {
        if (cudaMalloc(reinterpret_cast<void **>(&levels), n * sizeof(int32_t)) != cudaSuccess)
            reportError("cudaMalloc failed");
    }
    void release()
    {
        if (levels) cudaFree(levels);
        levels = nullptr;
        graph.free();
    }
    bw_launch_config cfg() const
    {
        return bw_launch_config{0, 0, static_cast<uint32_t>(warp), static_cast<uint32_t>(chunk)};
    }
    // The launch of `variant`: -w / -c when given, else the autotuner's
    // configuration for this graph (ImplementationTemplate.hpp:431-436 fixes
    // 32 / 32 instead)
    bw_launch_config cfg_for(int variant) const
    {
        if (warp || chunk) return cfg();
        return tuned_config("bfs", bw_bfs_variant_name(variant), graph.host);
    }
    void write(std::ofstream &out)
    {
        const uint64_t n = graph.view.vertex_count;
        std::vector<int32_t> h(n);
        Timer rt("resultTransfer");
        rt.start();
        if (cudaMemcpy(h.data(), levels, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            reportError("cudaMemcpy failed");
        rt.stop();
        for (uint64_t i = 0; i < n; i++) out << i << "\t" << h[i] << "\n";
    }
};

class BfsImplementation : public ImplementationBase {
  public:
    explicit BfsImplementation(int variant) : variant_(variant)
    {
        options.add('r', "root", "NUM", run_.root, "Starting vertex for BFS.");
        const std::string name = bw_bfs_variant_name(variant);
        if (name.rfind("vertex-push-warp", 0) == 0 || name.rfind("vertex-pull-warp", 0) == 0)
            add_warp_options();
    }

  protected:
    void add_warp_options()
    {
        options.add('w', "warp", "NUM", run_.warp, "Virtual warp size for warp variants.");
        options.add('c', "chunk", "NUM", run_.chunk, "Work chunk size for warp variants.");
    }
    void loadGraph(const std::string &file) override
    {
        Timer t("graphTransfer");
        t.start();
        run_.graph.load(file, bw_bfs_variant_reps(variant_) | 1);
        t.stop();
    }
    void freeGraph() override { run_.release(); }

    void runImplementation(std::ofstream &out) override
    {
        const uint64_t n = run_.graph.view.vertex_count;
        if (run_.root >= n) return;
        run_.alloc(n);
        Timer comp("computation");
        std::vector<bw_bfs_level_stats> stats(std::min<uint64_t>(n + 1, 1u << 20));
        bw_launch_config cfg = run_.cfg_for(variant_);
        for (size_t i = 0; i < run_count; i++) {
            bw_bfs_result res{};
            comp.start();
            check_bw(bw_bfs_run_schedule(shared_context(), &run_.graph.view, &variant_, 1, run_.root, run_.levels,
                                         &cfg, 0, 1, &res, stats.data(), static_cast<uint32_t>(stats.size()),
                                         nullptr),
                     "bfs");
            comp.stop();
            for (uint32_t L = 0; L < res.level_count && L < stats.size(); L++)
                Timer(std::to_string(L) + ":bfsLevel").record_ns(stats[L].device_ms * 1e6);
        }
        run_.write(out);
    }

    int variant_;
    BfsRun run_;
};

// `switch`: per-level variant choice by a predictor .so (bfs/bfs.cpp:83-106).
// Beside the reference's four step properties (setProps, bfs/bfs.cpp:43-49)
// it publishes the frontier's out-edge volume and log-degree moments, the
// out-edges already visited and the depth, which the learned predictor reads.
class BfsSwitch : public ImplementationBase, public SwitchBase {
  public:
    BfsSwitch() : SwitchBase(options, true)
    {
        options.add('r', "root", "NUM", run_.root, "Starting vertex for BFS.");
        abs_frontier_ = &add_algo_prop("frontier abs");
        rel_frontier_ = &add_algo_prop("frontier rel");
        abs_visited_ = &add_algo_prop("visited abs");
        rel_visited_ = &add_algo_prop("visited rel");
        frontier_edges_ = &add_algo_prop("frontier edges");
        log_sum_ = &add_algo_prop("frontier log degree sum");
        log_sq_sum_ = &add_algo_prop("frontier log degree square sum");
        log_max_ = &add_algo_prop("frontier log degree max");
        visited_edges_ = &add_algo_prop("visited edges");
        depth_ = &add_algo_prop("depth");
    }

  protected:
    void prepareRun() override
    {
        setup_switch([](const std::string &n) { return bw_bfs_variant_lookup(n.c_str()); }, "edge-list");
    }
    void cleanupRun() override { close(); }
    void loadGraph(const std::string &file) override
    {
        Timer t("graphTransfer");
        t.start();
        run_.graph.load(file, 63);
        t.stop();
        set_graph_props(run_.graph.host);
    }
    void freeGraph() override { run_.release(); }

    void runImplementation(std::ofstream &out) override
    {
        const uint64_t n = run_.graph.view.vertex_count;
        if (run_.root >= n) return;
        run_.alloc(n);
        Timer comp("computation");
        bw_launch_config cfg{};
        for (size_t i = 0; i < run_count; i++) {
            check_bw(bw_bfs_init(shared_context(), n, run_.root, run_.levels, nullptr), "bfs init");
            comp.start();
            *abs_frontier_ = 1;
            *rel_frontier_ = 1.0 / static_cast<double>(n);
            *abs_visited_ = 0;
            *rel_visited_ = 0;
            *visited_edges_ = 0;
            *depth_ = 0;
            set_frontier_stats(-1);
            int variant = predict_initial();
            cfg = picked_config(run_.cfg_for(variant), is_warp(variant));
            uint32_t frontier = 1;
            int32_t depth = 0;
            do {
                Timer lt(std::to_string(depth) + ":bfsLevel");
                lt.start();
                check_bw(bw_bfs_level(shared_context(), &run_.graph.view, variant, run_.levels, depth, &cfg,
                                      &frontier, nullptr),
                         "bfs level");
                lt.stop();
                depth++;
                if (frontier) {
                    // setProps (bfs/bfs.cpp:43-49)
                    *abs_visited_ = abs_visited_->get() + abs_frontier_->get();
                    *rel_visited_ = abs_visited_->get() / static_cast<double>(n);
                    *abs_frontier_ = frontier;
                    *rel_frontier_ = abs_frontier_->get() / static_cast<double>(n);
                    *visited_edges_ = visited_edges_->get() + frontier_edges_->get();
                    *depth_ = depth;
                    set_frontier_stats(depth - 1);
                    int next = predict();
                    if (next >= 0) {
                        variant = next;
                        cfg = picked_config(run_.cfg_for(variant), is_warp(variant));
                    }
                }
            } while (frontier);
            comp.stop();
        }
        run_.write(out);
    }

    static bool is_warp(int variant)
    {
        const std::string name = bw_bfs_variant_name(variant);
        return name.rfind("vertex-push-warp", 0) == 0 || name.rfind("vertex-pull-warp", 0) == 0;
    }

    // Statistics of the frontier the level at `depth` found (-1: {root}).
    void set_frontier_stats(int32_t depth)
    {
        bw_bfs_level_stats st{};
        check_bw(bw_bfs_frontier_stats(shared_context(), &run_.graph.view, run_.root, depth, &st, nullptr),
                 "frontier statistics");
        *frontier_edges_ = static_cast<double>(st.frontier_edges);
        *log_sum_ = st.log_degree_sum;
        *log_sq_sum_ = st.log_degree_sq_sum;
        *log_max_ = st.log_degree_max;
    }

    BfsRun run_;
    prop_ref *abs_frontier_, *rel_frontier_, *abs_visited_, *rel_visited_;
    prop_ref *frontier_edges_, *log_sum_, *log_sq_sum_, *log_max_, *visited_edges_, *depth_;
};

}  // namespace

extern "C" register_algorithm_t registerCUDA;
extern "C" void registerCUDA(Algorithm &result)
{
    INITIALISE_ALGORITHM(result);
    for (int v = 0; v < bw_bfs_variant_count(); v++)
        result.addImplementation(bw_bfs_variant_name(v), std::make_unique<BfsImplementation>(v));
    result.addImplementation("switch", std::make_unique<BfsSwitch>());
}
