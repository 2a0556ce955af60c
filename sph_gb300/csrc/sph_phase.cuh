// Named step phases: an NVTX range per phase (seen by Nsight Systems and by
// ncu's NVTX filters) and, while profiling is on, CUDA-event times per phase
// on the launching stream.
//
// The names are those of the reference's wall-clock phase timers
// (Simulation::startCounting / stopCounting, TimeManager.h:68-94) without
// their padding: DFSPHSolver.cpp:43-101 ("npForces", "Density solver",
// "Boundary handling", "Fill grid", "Neigh search", "Densities",
// "Alpha factor", "Divergence solver"), PCISPHSolver.cpp:26-67 (+ "Pressure
// solver", "Integration"), WCSPHSolver.cpp:20-64 ("Pressures",
// "Pressure force", "NPForces", "Integratio", "Boundary Handling", spelled as
// there) and Simulation.cpp:158 ("Step computation", one whole step).  A
// phase whose kernels fuse several of the reference's phases joins their
// names with '+' ("Neigh search+Densities+Alpha factor": the pair-list build
// also forms densities and alpha factors), so that a side-by-side table sums
// the reference's rows.  Inside a graph capture nothing is recorded: a graph
// step is one "Step computation" range.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace sph {

class PhaseLog {
public:
    PhaseLog() = default;
    PhaseLog(const PhaseLog&) = delete;
    PhaseLog& operator=(const PhaseLog&) = delete;
    ~PhaseLog()
    {
        for (auto& m : pending_) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
        for (auto e : spare_) cudaEventDestroy(e);
    }

    cudaEvent_t take()
    {
        if (!spare_.empty()) { cudaEvent_t e = spare_.back(); spare_.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void add(const char* name, cudaEvent_t a, cudaEvent_t b) { pending_.push_back({name, a, b}); }

    // "name<TAB>count<TAB>total_ms" per phase, in first-seen order, for the
    // phases timed since the previous call; returns the text length or a
    // negative CUDA error.  The stream must be synchronised by the caller.
    int report(char* buf, size_t len)
    {
        std::vector<const char*> names;
        std::vector<double> ms;
        std::vector<unsigned long long> cnt;
        for (auto& m : pending_) {
            float t = 0.f;
            const cudaError_t e = cudaEventElapsedTime(&t, m.a, m.b);
            if (e != cudaSuccess) return -(int)e;
            size_t k = 0;
            while (k < names.size() && std::strcmp(names[k], m.name) != 0) ++k;
            if (k == names.size()) { names.push_back(m.name); ms.push_back(0.0); cnt.push_back(0); }
            ms[k] += t;
            cnt[k] += 1;
            spare_.push_back(m.a);
            spare_.push_back(m.b);
        }
        pending_.clear();
        std::string out;
        char line[160];
        for (size_t k = 0; k < names.size(); ++k) {
            std::snprintf(line, sizeof line, "%s\t%llu\t%.6f\n", names[k], cnt[k], ms[k]);
            out += line;
        }
        if (buf && len) {
            std::strncpy(buf, out.c_str(), len - 1);
            buf[len - 1] = 0;
        }
        return (int)out.size();
    }

private:
    struct Mark {
        const char* name;   // a string literal
        cudaEvent_t a, b;
    };
    std::vector<Mark> pending_;
    std::vector<cudaEvent_t> spare_;
};

// One phase: an NVTX range for the scope and, when TIMED, a pair of events
// recorded on STREAM around it.  Inactive while a graph is being captured.
class Phase {
public:
    Phase(PhaseLog& log, const char* name, cudaStream_t stream, bool capturing, bool timed)
        : log_(log), name_(name), stream_(stream), on_(!capturing), timed_(!capturing && timed)
    {
        if (!on_) return;
        nvtxRangePushA(name);
        if (timed_) {
            a_ = log_.take();
            cudaEventRecord(a_, stream_);
        }
    }
    ~Phase()
    {
        if (!on_) return;
        if (timed_) {
            cudaEvent_t b = log_.take();
            cudaEventRecord(b, stream_);
            log_.add(name_, a_, b);
        }
        nvtxRangePop();
    }
    Phase(const Phase&) = delete;
    Phase& operator=(const Phase&) = delete;

private:
    PhaseLog& log_;
    const char* name_;
    cudaStream_t stream_;
    bool on_, timed_;
    cudaEvent_t a_ = nullptr;
};

}  // namespace sph
