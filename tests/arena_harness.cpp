// CPU harness for rmq_arena.h: reads commands from stdin and prints the
// result of each, so the test can check the arena against a model.
//   i SIZE        init
//   a BYTES       alloc  -> "ok OFF" or "full"
//   r OFF BYTES   release
//   f             free ranges -> "free N off len off len ..."
//   v EXCEPT N (resident ready pins last_use) x N
//                 eviction choice -> "victim I" (or "victim none")
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "rmq_arena.h"

struct Entry {
    bool resident, ready;
    int pins;
    uint64_t last_use;
};

int main() {
    rmq::Arena arena;
    std::string cmd;
    while (std::cin >> cmd) {
        if (cmd == "i") {
            uint64_t size;
            std::cin >> size;
            arena.init(size);
        } else if (cmd == "a") {
            uint64_t bytes, off = 0;
            std::cin >> bytes;
            if (arena.alloc(bytes, &off)) std::printf("ok %llu\n", (unsigned long long)off);
            else std::printf("full\n");
        } else if (cmd == "r") {
            uint64_t off, bytes;
            std::cin >> off >> bytes;
            arena.release(off, bytes);
        } else if (cmd == "v") {
            uint64_t except, n;
            std::cin >> except >> n;
            std::vector<Entry> arrays(n);
            for (auto& e : arrays) {
                int res, rdy;
                std::cin >> res >> rdy >> e.pins >> e.last_use;
                e.resident = res != 0;
                e.ready = rdy != 0;
            }
            const uint64_t v = rmq::lru_victim(arrays, except);
            if (v == ~uint64_t(0)) std::printf("victim none\n");
            else std::printf("victim %llu\n", (unsigned long long)v);
        } else if (cmd == "f") {
            const auto& fr = arena.free_ranges();
            std::printf("free %zu", fr.size());
            for (const auto& kv : fr) std::printf(" %llu %llu", (unsigned long long)kv.first, (unsigned long long)kv.second);
            std::printf("\n");
        }
    }
    return 0;
}
