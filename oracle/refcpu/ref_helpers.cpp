/*
 * The two host helpers the reference uses from helper.cu (printArray,
 * copyArray; helper.cu:3-60), which does not compile under GCC 13
 * (helper.cu:86 streams std::cout into an ostream).  Same output format:
 * each value followed by a space, one row per line.
 *
 * Test infrastructure only.
 */
#include <iostream>

template <class T>
static void print_array(T *array, int dim1, int dim2, std::ostream &stream) {
  for (int i = 0; i < dim1; ++i) {
    for (int j = 0; j < dim2; ++j) stream << array[i * dim2 + j] << " ";
    stream << std::endl;
  }
}
void printArray(float *a, int d1, int d2, std::ostream &s) { print_array(a, d1, d2, s); }
void printArray(int *a, int d1, int d2, std::ostream &s) { print_array(a, d1, d2, s); }
void printArray(bool *a, int d1, int d2, std::ostream &s) { print_array(a, d1, d2, s); }
void printArray(char *a, int d1, int d2, std::ostream &s) { print_array(a, d1, d2, s); }
void copyArray(float *to, float *from, int length) {
  for (int i = 0; i < length; ++i) to[i] = from[i];
}
