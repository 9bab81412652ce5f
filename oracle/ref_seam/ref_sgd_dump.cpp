// Replaces the reference's sgd_train (sgd_Kernel.h:24-38) with a dump of the
// schedule that block_problem hands over: num_parallel, max_parallel,
// num_bs[] and, per slot, block id, nnz, coe weights (as hex floats) and the
// entries' coordinates in block order.  Test infrastructure only.
#include "tensor_SGD.h"
#include <cstdio>

extern std::string g_dump_dir;

void sgd_train(const T_node*, int train_nnz, const T_node*, int, double*, double*, double*,
               int num_parallel, int max_parallel, LF_node*, int*, double, int* num_bs,
               b_node* bs, int num_scheduled_bs) {
    FILE* f = fopen((g_dump_dir + "/schedule.txt").c_str(), "w");
    fprintf(f, "num_parallel %d\nmax_parallel %d\nscheduled %d\ntrain_nnz %d\n", num_parallel,
            max_parallel, num_scheduled_bs, train_nnz);
    int groups = num_parallel > 1 ? num_parallel - 1 : 0;
    fprintf(f, "num_bs");
    for (int i = 0; i < groups; i++) fprintf(f, " %d", num_bs[i]);
    fprintf(f, "\n");
    for (int k = 0; k < num_scheduled_bs; k++) {
        fprintf(f, "slot %d %d %d %a %a %a\n", k, bs[k].id, bs[k].block_num, bs[k].coe_x,
                bs[k].coe_y, bs[k].coe_z);
        for (int i = 0; i < bs[k].block_num; i++)
            fprintf(f, "%d %d %d\n", bs[k].x[i], bs[k].y[i], bs[k].z[i]);
    }
    fclose(f);
}
