// Harness around the reference's own CPU Bellman-Ford (src/sssp/base-perk/SSSP.cpp:88-119).
// TEST INFRASTRUCTURE ONLY: oracle/build.py compiles it together with that reference
// source file, where it lies in the reference tree, into oracle/_ref/ref-bf.  The
// fixtures in tests/golden/ come from it.
//
//   ref-bf <dataset_dir> <source> <out_dist.bin> [seeds.bin]
//
// Reads <dataset_dir>/origin/{vlist,elist,wlist}.bin through the reference Graph class,
// sets dist[source] = 0, lowers dist[v] to w for every (v, w) int32 pair of seeds.bin,
// runs Bellman_ford from the frontier seeds + source (the sssp-purn launch order,
// src/sssp/purn/Main.cu:72-90,160-181) and writes the int32 distances.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Graph.h"

extern Graph graph;
void Bellman_ford(ValueType* distance, int* global_ft, int global_ft_cnt);

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: ref-bf <dir> <source> <out> [seeds.bin]\n");
        return 2;
    }
    graph.Graphinit(argv[1]);
    const int s = atoi(argv[2]);
    std::vector<int> dist(graph.vert_num, 1999999999);
    std::vector<int> frontier;
    if (argc > 4) {
        FILE* fp = fopen(argv[4], "rb");
        if (!fp) return 3;
        int vw[2];
        while (fread(vw, sizeof(int), 2, fp) == 2) {
            if (vw[1] < dist[vw[0]]) dist[vw[0]] = vw[1];
            frontier.push_back(vw[0]);
        }
        fclose(fp);
    }
    dist[s] = 0;
    frontier.push_back(s);
    Bellman_ford(dist.data(), frontier.data(), (int)frontier.size());
    FILE* out = fopen(argv[3], "wb");
    if (!out) return 4;
    fwrite(dist.data(), sizeof(int), dist.size(), out);
    fclose(out);
    return 0;
}
