// Driver for the reference blocking/schedule code (block.cu:1233-1287) on the
// CPU.  Reads 0-based "x y z value" lines, shuffles them exactly as the
// reference main does (main.cpp:303-306: std::mt19937(42) + std::shuffle),
// dumps the shuffled order, and calls block_problem.  block_problem writes
// block_parallel.txt and then calls sgd_train, which ref_sgd_dump.cpp replaces
// with a schedule dump.  Test infrastructure only.
//
// usage: ref_block <in.txt> <I> <J> <K> <block_s> <pss> <outdir> <dataset> <train_rate>
#include "tensor_SGD.h"
#include "block.h"
#include <algorithm>
#include <cstdio>

std::string g_dump_dir;

int main(int argc, char** argv) {
    if (argc != 10) {
        fprintf(stderr, "usage: %s in I J K block_s pss outdir dataset train_rate\n", argv[0]);
        return 2;
    }
    I = atoi(argv[2]);
    J = atoi(argv[3]);
    K = atoi(argv[4]);
    block_s = atoi(argv[5]);
    parallel_sequence_size = atoi(argv[6]);
    output_root = argv[7];
    dataset_name = argv[8];
    double rate = atof(argv[9]);
    g_dump_dir = output_root;
    std::vector<T_node> v;
    FILE* f = fopen(argv[1], "r");
    if (!f) return 3;
    T_node t;
    while (fscanf(f, "%d %d %d %lf", &t.x, &t.y, &t.z, &t.rate) == 4) v.push_back(t);
    fclose(f);
    if (v.size() > 1) {
        std::mt19937 rng(42);
        std::shuffle(v.begin(), v.end(), rng);
    }
    FILE* so = fopen((g_dump_dir + "/shuffled.txt").c_str(), "w");
    for (size_t i = 0; i < v.size(); i++) fprintf(so, "%d %d %d\n", v[i].x, v[i].y, v[i].z);
    fclose(so);
    double* a = new double[(size_t)I * r];
    double* b = new double[(size_t)J * r];
    double* c = new double[(size_t)K * r];
    block_problem(v.data(), (int)v.size(), NULL, 0, a, b, c, rate);
    return 0;
}
