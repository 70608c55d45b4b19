// Stage timers: CUDA events recorded on the solver's stream around each
// stage, resolved and accumulated at the end of every step.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

namespace ibm {

struct Prof {
    bool on = false;
    cudaStream_t s = nullptr;
    struct Rec {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    std::map<std::string, std::pair<long, double>> total;

    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    int begin(const char *name) {
        if (!on) return -1;
        Rec r{name, get(), get()};
        cudaEventRecord(r.a, s);
        pending.push_back(r);
        return (int)pending.size() - 1;
    }
    void end(int idx) {
        if (idx < 0) return;
        cudaEventRecord(pending[idx].b, s);
    }
    void flush() {
        if (pending.empty()) return;
        cudaStreamSynchronize(s);
        for (auto &r : pending) {
            float ms = 0;
            cudaEventElapsedTime(&ms, r.a, r.b);
            auto &t = total[r.name];
            t.first += 1;
            t.second += ms;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.clear();
    }
    void reset() {
        flush();
        total.clear();
    }
    ~Prof() {
        for (auto &r : pending) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace ibm
