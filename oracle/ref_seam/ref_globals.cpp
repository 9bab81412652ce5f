// Seam for running the reference's unmodified block.cu on the CPU.
// Defines the configuration globals that the reference declares in
// tensor_SGD.h:25-42 (and defines in tensor_SGD.cu:24-41), with the same
// defaults, so that block.cu links without the reference's tensor_SGD.cu.
// Test infrastructure only: built into oracle/_ref by oracle/Makefile.
#include "tensor_SGD.h"

int I = 144;
int J = 288;
int K = 168;
int epochs = 1000;
int r = 16;
double lr = 0.005;
double reg = 0.0005;
int block_s = 2048;
int thread_size = 512;
int flag_lockfree = 0;
int flag_preproccess = 1;
int parallel_sequence_size = 8;
int requested_gpu_count = 4;
queue<double> num1;
string dataset_name = "tensor";
string output_root = "output";
double train_rate = 0.8;
