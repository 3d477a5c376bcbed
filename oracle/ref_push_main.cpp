// Harness around the reference's own CPU forward push (src/ppr/w-purn-perk/PPR.cpp:178-233).
// TEST INFRASTRUCTURE ONLY: oracle/build.py compiles it together with that reference
// source file, where it lies in the reference tree, into oracle/_ref/ref-push.  The
// fixtures in tests/golden/ come from it.
//
//   ref-push <dataset_dir> <source> <rmax> <out_prefix>
//
// Reads <dataset_dir>/origin/{vlist,elist,flist}.bin through the reference Graph class,
// sets graph.rmax, applies the base-program init (residual 1 and pagerank alpha on the
// source, src/ppr/base/Main.cu:146-150), runs forward_push from {source} and writes
// <out_prefix>.pr.bin and <out_prefix>.res.bin (float32).  forward_push allocates its
// message and flag arrays without initialising them, so the harness makes the
// allocator serve every allocation above 4 KiB from fresh zero-filled pages.
#include <malloc.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "Graph.h"

extern Graph graph;
void forward_push(ValueType* reserve, ValueType* residue, Vertex* global_ft_1, Vertex global_ft1_cnt);
extern const ValueType alpha;

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: ref-push <dir> <source> <rmax> <out_prefix>\n");
        return 2;
    }
    mallopt(M_MMAP_THRESHOLD, 4096);
    graph.Graphinit(argv[1]);
    const int s = atoi(argv[2]);
    graph.rmax = (ValueType)atof(argv[3]);
    std::vector<ValueType> reserve(graph.vert_num, 0.0f), residue(graph.vert_num, 0.0f);
    residue[s] = 1.0f;
    reserve[s] += alpha * residue[s];
    int ft = s;
    forward_push(reserve.data(), residue.data(), &ft, 1);
    const std::string pre = argv[4];
    FILE* f1 = fopen((pre + ".pr.bin").c_str(), "wb");
    FILE* f2 = fopen((pre + ".res.bin").c_str(), "wb");
    if (!f1 || !f2) return 4;
    fwrite(reserve.data(), sizeof(ValueType), reserve.size(), f1);
    fwrite(residue.data(), sizeof(ValueType), residue.size(), f2);
    fclose(f1);
    fclose(f2);
    return 0;
}
