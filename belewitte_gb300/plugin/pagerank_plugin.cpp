// libpagerankkernel.so: the PageRank algorithm library kernel-runner loads.
// Registers the reference's ten implementation names
// (pagerank/pagerank.cpp:205-351), the GB300 variants and `switch`.
//
// Run semantics follow PageRank::runImplementation
// (pagerank/pagerank.cpp:74-171): a fixed iteration count (100 in the
// reference; `-i/--iterations` here), `computation`, `0:computation` and
// `resultTransfer` timers, and the two output forms: --validate prints
// `vertex \t rank` with digits10 + 1 significant digits, otherwise the
// vertex ids ordered by rank with the low 16 mantissa bits masked and each
// 1000-entry bucket re-sorted by id (pagerank.cpp:142-168).
#include <cmath>
#include <algorithm>
#include <cstring>
#include <iomanip>
#include <limits>
#include <cuda_runtime_api.h>

#include "framework.hpp"
#include "switching.hpp"

namespace {

void write_ranks(std::ofstream &out, const std::vector<float> &pr, bool validate)
{
    auto old = out.imbue(std::locale("C"));
    if (validate) {
        out << std::setprecision(std::numeric_limits<float>::digits10 + 1);
        for (size_t i = 0; i < pr.size(); i++) out << i << "\t" << pr[i] << "\n";
    } else {
        const uint32_t mask = ~((1u << 16) - 1u);
        std::vector<std::pair<float, size_t>> buckets;
        buckets.reserve(pr.size());
        for (size_t i = 0; i < pr.size(); i++) {
            uint32_t bits;
            std::memcpy(&bits, &pr[i], 4);
            bits &= mask;
            float v;
            std::memcpy(&v, &bits, 4);
            buckets.emplace_back(v, i);
        }
        std::stable_sort(buckets.begin(), buckets.end());
        const size_t bucket = 1000;
        for (size_t i = 0; i < buckets.size(); i += bucket) {
            const size_t hi = std::min(i + bucket, buckets.size() - 1);
            std::stable_sort(buckets.begin() + static_cast<long>(i), buckets.begin() + static_cast<long>(hi),
                             [](const auto &a, const auto &b) { return a.second < b.second; });
        }
        for (const auto &p : buckets) out << p.second << "\n";
    }
    out.imbue(old);
}

class PageRankBase : public ImplementationBase {
  protected:
    PageRankBase()
    {
        options.add('i', "iterations", "NUM", iterations_, "Number of PageRank iterations (reference: 100).");
    }
    void loadGraph(const std::string &file) override
    {
        Timer t("graphTransfer");
        t.start();
        graph_.load(file, reps_);
        t.stop();
        after_load();
    }
    virtual void after_load() {}
    // The launch configuration of `variant`: the -w/-c options when given,
    // else the autotuner's configuration for this graph
    // (ImplementationTemplate.hpp:431-436 fixes 32 / 32 instead).
    virtual bw_launch_config config_for(int variant)
    {
        if (warp_ || chunk_) return bw_launch_config{0, 0, static_cast<uint32_t>(warp_), static_cast<uint32_t>(chunk_)};
        return tuned_config("pagerank", bw_pagerank_variant_name(variant), graph_.host);
    }
    void freeGraph() override
    {
        if (ranks_) cudaFree(ranks_);
        ranks_ = nullptr;
        graph_.free();
    }
    void run(std::ofstream &out, std::function<int()> pick)
    {
        const uint64_t n = graph_.view.vertex_count;
        if (cudaMalloc(reinterpret_cast<void **>(&ranks_), n * 4) != cudaSuccess) reportError("cudaMalloc failed");
        Timer comp("computation"), step("0:computation");
        for (size_t i = 0; i < run_count; i++) {
            const int variant = pick();
            const bw_launch_config cfg = config_for(variant);
            bw_pagerank_result res{};
            comp.start();
            check_bw(bw_pagerank_run(shared_context(), &graph_.view, variant, iterations_, ranks_, &cfg, 0, &res,
                                     nullptr, nullptr),
                     "pagerank");
            comp.stop();
            step.record_ns(res.device_ms * 1e6);
        }
        std::vector<float> h(n);
        Timer rt("resultTransfer");
        rt.start();
        if (cudaMemcpy(h.data(), ranks_, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            reportError("cudaMemcpy failed");
        rt.stop();
        write_ranks(out, h, validate);
    }

    unsigned iterations_ = 100;
    size_t warp_ = 0, chunk_ = 0;      // -w / -c; 0: tuned, else the library's 32 / 32
    int reps_ = 63;
    LoadedGraph graph_;
    float *ranks_ = nullptr;
};

class PageRankImplementation : public PageRankBase {
  public:
    explicit PageRankImplementation(int variant) : variant_(variant)
    {
        reps_ = bw_pagerank_variant_reps(variant);
        const std::string name = bw_pagerank_variant_name(variant);
        if (name.find("-warp") != std::string::npos) {
            options.add('w', "warp", "NUM", warp_, "Virtual warp size for warp variants.");
            options.add('c', "chunk", "NUM", chunk_, "Work chunk size for warp variants.");
        }
    }

  protected:
    void runImplementation(std::ofstream &out) override { run(out, [this] { return variant_; }); }
    int variant_;
};

// `switch`: the predictor picks one variant per run from the graph
// properties (pagerank/pagerank.cpp:98-100 calls predictInitial only).
// Beside the reference's graph properties it publishes the in-degree log
// moments (sum, sum of squares and max of log2(1 + in-degree)), which the
// learned PageRank predictor reads.
class PageRankSwitch : public PageRankBase, public SwitchBase {
  public:
    PageRankSwitch() : SwitchBase(options, false)
    {
        log_sum_ = &add_graph_prop("in log degree sum");
        log_sq_sum_ = &add_graph_prop("in log degree square sum");
        log_max_ = &add_graph_prop("in log degree max");
    }

  protected:
    void prepareRun() override
    {
        setup_switch([](const std::string &n) { return bw_pagerank_variant_lookup(n.c_str()); }, "edge-list");
    }
    void cleanupRun() override { close(); }
    void after_load() override
    {
        set_graph_props(graph_.host);
        const bw_host_graph &h = graph_.host;
        const uint32_t *off = h.rev_vertices ? h.rev_vertices : h.fwd_vertices;
        double ls = 0.0, lq = 0.0, lm = 0.0;
        for (uint64_t v = 0; off && v < h.vertex_count; v++) {
            const double l = std::log2(1.0 + static_cast<double>(off[v + 1] - off[v]));
            ls += l;
            lq += l * l;
            lm = std::max(lm, l);
        }
        *log_sum_ = ls;
        *log_sq_sum_ = lq;
        *log_max_ = lm;
    }
    prop_ref *log_sum_, *log_sq_sum_, *log_max_;
    void runImplementation(std::ofstream &out) override { run(out, [this] { return predict_initial(); }); }
    // a warp variant runs with the warp and chunk sizes its predictor slot gives
    bw_launch_config config_for(int variant) override
    {
        const bool warp = std::string(bw_pagerank_variant_name(variant)).find("-warp") != std::string::npos;
        return picked_config(PageRankBase::config_for(variant), warp);
    }
};

}  // namespace

extern "C" register_algorithm_t registerCUDA;
extern "C" void registerCUDA(Algorithm &result)
{
    INITIALISE_ALGORITHM(result);
    for (int v = 0; v < bw_pagerank_variant_count(); v++)
        result.addImplementation(bw_pagerank_variant_name(v), std::make_unique<PageRankImplementation>(v));
    result.addImplementation("switch", std::make_unique<PageRankSwitch>());
}
