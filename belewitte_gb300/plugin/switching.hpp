// Predictor-driven variant switching of the plugin surface
// (SwitchImplementation, ImplementationTemplate.hpp:545-908).
//
// A predictor is a shared library exporting, unmangled (extern "C") with
// C++ types as the reference's exported decision trees do
// (benchmark-analysis src/Predictor/Raw.hs:56-139):
//   int32_t lookup();
//   std::map<std::string, std::reference_wrapper<double>> propNames;
//   std::vector<std::tuple<std::string,int64_t,size_t,size_t,size_t>> implNames;
//   int32_t default_impl;
// Properties named in propNames are re-pointed at the predictor's storage,
// so setting them feeds lookup(); every other property gets storage of its
// own (as the reference's setupLogging gives the logged ones,
// ImplementationTemplate.hpp:845-867), so that it holds its value.  Without a model the switch runs
// `edge-list` and only logs (ImplementationTemplate.hpp:709-720).
// Log lines: graph:NAME:VALUE, step:N:NAME:VALUE, prediction:N:ID
// (ImplementationTemplate.hpp:829-876).
#pragma once

#include <dlfcn.h>

#include <map>
#include <set>

#include "framework.hpp"

class SwitchBase {
  public:
    using impl_tuple = std::tuple<std::string, int64_t, size_t, size_t, size_t>;

    SwitchBase(Options &opts, bool per_step) : per_step_(per_step)
    {
        opts.add('m', "model", "FILE", model_, "Prediction model to use.");
        opts.add('l', "log", "FILE", log_file_, "Where to log properties.");
        for (const char *kind : {"abs", "in", "out"}) {
            for (const char *stat : {"min ", "lower quantile ", "mean ", "median ", "upper quantile ", "max ",
                                     "stddev "})
                add_graph_prop(std::string(stat) + kind + " degree");
        }
        add_graph_prop("vertex count");
        add_graph_prop("edge count");
    }
    virtual ~SwitchBase() { close(); }

  protected:
    std::map<std::string, std::unique_ptr<prop_ref>> graph_props_, algo_props_;

    prop_ref &add_graph_prop(const std::string &name)
    { return *(graph_props_[name] = std::make_unique<prop_ref>()); }
    prop_ref &add_algo_prop(const std::string &name)
    { return *(algo_props_[name] = std::make_unique<prop_ref>()); }

    // Fill the graph-level properties (SwitchImplementation::loadGraph,
    // ImplementationTemplate.hpp:622-649).
    void set_graph_props(const bw_host_graph &g)
    {
        const char *kinds[3] = {"abs", "in", "out"};
        const char *stats[7] = {"min ", "lower quantile ", "mean ", "median ", "upper quantile ", "max ", "stddev "};
        for (int k = 0; k < 3; k++) {
            double out[7];
            check_bw(bw_degree_statistics(&g, k, out), "degree statistics");
            for (int s = 0; s < 7; s++) *graph_props_[std::string(stats[s]) + kinds[k] + " degree"] = out[s];
        }
        *graph_props_["vertex count"] = static_cast<double>(g.vertex_count);
        *graph_props_["edge count"] = static_cast<double>(g.edge_count);
    }

    // Map the predictor's implementation table onto variant ids.
    void setup_switch(std::function<int(const std::string &)> lookup_variant, const std::string &default_name)
    {
        impls_.clear();
        ids_.clear();
        bound_.clear();
        storage_.clear();
        last_ = -1;
        step_ = 0;
        if (!model_.empty()) {
            handle_ = dlopen(model_.c_str(), RTLD_NOW);
            if (!handle_) reportError(std::string("dlopen() failed: ") + model_ + "\n" + dlerror());
            lookup_ = reinterpret_cast<int32_t (*)()>(sym("lookup"));
            auto &names = *reinterpret_cast<std::vector<impl_tuple> *>(sym("implNames"));
            auto &props = *reinterpret_cast<std::map<std::string, std::reference_wrapper<double>> *>(sym("propNames"));
            default_ = *reinterpret_cast<int32_t *>(sym("default_impl"));
            bool missing = false;
            for (auto &p : props) {
                auto g = graph_props_.find(p.first);
                auto a = algo_props_.find(p.first);
                if (g != graph_props_.end()) *g->second = p.second;
                else if (a != algo_props_.end()) *a->second = p.second;
                else { std::cerr << "Missing property: " << p.first << std::endl; missing = true; }
            }
            impls_.resize(names.size());
            ids_.resize(names.size());
            warp_.assign(names.size(), 0);
            chunk_.assign(names.size(), 0);
            for (auto &t : names) {
                const size_t idx = std::get<2>(t);
                const int v = lookup_variant(std::get<0>(t));
                if (v < 0 || idx >= names.size()) {
                    std::cerr << "Missing implementation: " << std::get<0>(t) << std::endl;
                    missing = true;
                    continue;
                }
                impls_[idx] = v;
                ids_[idx] = std::get<1>(t);
                // the warp and chunk sizes the slot runs its warp kernels
                // with (ImplementationTemplate.hpp:806-816: setWarpConfig)
                warp_[idx] = static_cast<uint32_t>(std::get<3>(t));
                chunk_[idx] = static_cast<uint32_t>(std::get<4>(t));
            }
            if (missing) reportError("Missing properties/implementations!");
            for (auto &p : props) bound_.insert(p.first);
        } else {
            lookup_ = nullptr;
            default_ = 0;
            impls_.push_back(lookup_variant(default_name));
            ids_.push_back(-1);
            warp_.assign(1, 0);
            chunk_.assign(1, 0);
        }
        for (auto *table : {&graph_props_, &algo_props_})
            for (auto &p : *table)
                if (!bound_.count(p.first)) *p.second = std::ref(storage_[p.first] = 0.0);
        if (!log_file_.empty()) {
            log_.open(log_file_);
            log_.imbue(std::locale("C"));
        }
    }

    int predict_initial()
    {
        step_ = 0;
        if (log_.is_open()) {
            for (auto &p : graph_props_) log_ << "graph:" << p.first << ":" << p.second->get() << "\n";
            log_algo();
        }
        int32_t r = lookup();
        last_ = r == -1 ? default_ : r;
        return impls_[static_cast<size_t>(last_)];
    }

    // Returns the variant for the next step, or -1 to keep the current one.
    int predict()
    {
        ++step_;
        if (log_.is_open()) log_algo();
        int32_t r = lookup();
        if (r != -1 && r != last_) {
            last_ = r;
            return impls_[static_cast<size_t>(r)];
        }
        return -1;
    }

    // The launch configuration of the implementation picked last: `base`
    // (the -w/-c options) with, for a warp variant, the warp and chunk sizes
    // the predictor's implNames entry gives it, as the reference applies
    // them to its warp kernels (setWarpConfig, ImplementationTemplate.hpp:
    // 806-816).  Logged as "config:<step>:<warp>:<chunk>".
    bw_launch_config picked_config(bw_launch_config base, bool warp_variant)
    {
        if (!warp_variant || !lookup_ || last_ < 0) return base;
        const uint32_t w = warp_[static_cast<size_t>(last_)], c = chunk_[static_cast<size_t>(last_)];
        if (w == 0 || c == 0) return base;
        base.warp_size = w;
        base.chunk_size = c;
        if (log_.is_open()) log_ << "config:" << step_ << ":" << w << ":" << c << "\n";
        return base;
    }

    void close()
    {
        if (handle_) { dlclose(handle_); handle_ = nullptr; }
        if (log_.is_open()) log_.close();
        for (auto &p : graph_props_) p.second->reset();
        for (auto &p : algo_props_) p.second->reset();
        bound_.clear();
        storage_.clear();
    }

  private:
    void *sym(const char *name)
    {
        void *p = dlsym(handle_, name);
        if (!p) reportError(std::string("dlsym() failed: ") + name);
        return p;
    }
    void log_algo()
    {
        for (auto &p : algo_props_) log_ << "step:" << step_ << ":" << p.first << ":" << p.second->get() << "\n";
    }
    int32_t lookup()
    {
        int32_t r = lookup_ ? lookup_() : -1;
        if (log_.is_open()) {
            int32_t shown = r == -1 ? (last_ == -1 ? default_ : last_) : r;
            log_ << "prediction:" << step_ << ":" << ids_[static_cast<size_t>(shown)] << "\n";
        }
        return r;
    }

    bool per_step_;
    std::string model_, log_file_;
    void *handle_ = nullptr;
    int32_t (*lookup_)() = nullptr;
    int32_t default_ = 0, last_ = -1;
    size_t step_ = 0;
    std::vector<int> impls_;
    std::vector<int64_t> ids_;
    std::vector<uint32_t> warp_, chunk_;       // implNames fields 3 and 4 per slot
    std::set<std::string> bound_;              // properties the predictor owns
    std::map<std::string, double> storage_;    // the others (map nodes do not move)
    std::ofstream log_;
};
