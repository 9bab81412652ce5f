// Replaces the reference's tensor_SGD (tensor_SGD.cu:55-90) for parity runs
// of the reference binary: the factors start from a file instead of
// std::random_device (tensor_SGD.cu:43-53), and the final factors that
// sgd_train copies back (sgd_Kernel.cu:1341-1343) are written to a file.
//   BTC_REF_INIT  binary doubles A[I*r], B[J*r], C[K*r] (required)
//   BTC_REF_DUMP  where to write the final factors in the same layout
// Test infrastructure only: linked with the reference's own main.cpp,
// block.cu and sgd_Kernel.cu by `make -C oracle refgpu`.
#include <cstdio>
#include <cstdlib>

#include "block.h"
#include "tensor_SGD.h"

void tensor_SGD(const vector<T_node>& train_entries, const vector<T_node>& test_entries)
{
    cout << "dataset=" << dataset_name << " dims=" << I << "x" << J << "x" << K
         << " train_nnz=" << train_entries.size() << " test_nnz=" << test_entries.size() << endl;
    double* a = new double[(size_t)I * r];
    double* b = new double[(size_t)J * r];
    double* c = new double[(size_t)K * r];
    const char* init = getenv("BTC_REF_INIT");
    FILE* f = init ? fopen(init, "rb") : NULL;
    if (!f) {
        cerr << "BTC_REF_INIT must name the initial factor file" << endl;
        exit(2);
    }
    size_t n = fread(a, 8, (size_t)I * r, f) + fread(b, 8, (size_t)J * r, f) + fread(c, 8, (size_t)K * r, f);
    fclose(f);
    if (n != (size_t)(I + J + K) * r) {
        cerr << "short initial factor file" << endl;
        exit(2);
    }
    block_problem(train_entries.data(), (int)train_entries.size(), test_entries.data(),
                  (int)test_entries.size(), a, b, c, train_rate);
    const char* dump = getenv("BTC_REF_DUMP");
    if (dump) {
        FILE* o = fopen(dump, "wb");
        fwrite(a, 8, (size_t)I * r, o);
        fwrite(b, 8, (size_t)J * r, o);
        fwrite(c, 8, (size_t)K * r, o);
        fclose(o);
    }
    delete[] a;
    delete[] b;
    delete[] c;
}
