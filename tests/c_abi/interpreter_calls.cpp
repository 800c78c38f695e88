// Links against libaces4gb300.so with the drop-in entry points declared the
// way the SIP interpreter sees them (tensor_ops_c_prototypes.h: scalars by
// C++ reference, extern "C" names of the Fortran bind(c) routines), and
// replays the interpreter's call sequences on host blocks:
//   handle_contraction (interpreter.cpp:1210-1262): get_contraction_ptrn_ then
//     tensor_block_contract__ on [d ids, l ids, r ids];
//   Block::transpose_copy (block.cpp:448-487): tensor_block_copy__ with the
//     O2N permutation and its sign slot;
//   tensor_block_add__ (d += s * scale).
// Input: a text file of cases written by the test (dims, labels, operands,
// expected results); every result must match bit for bit.  Exit status 0
// when all do.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

extern "C" {
void get_contraction_ptrn_(int& drank, int& lrank, int& rrank, int* aces_ptrn, int* my_ptrn, int& ierr);
void tensor_block_contract__(int&, int*, double*, int&, int*, double*, int&, int*, double*, int&, int*, int&);
void tensor_block_copy__(int&, int&, int*, int*, double*, double*, int&);
void tensor_block_add__(const int&, const int&, int*, double*, double*, const double&, int&);
const char* a4g_last_error(void);
}

static std::vector<int> read_ints(FILE* f) {
  int n = 0;
  if (fscanf(f, "%d", &n) != 1) exit(3);
  std::vector<int> v(n);
  for (int& x : v)
    if (fscanf(f, "%d", &x) != 1) exit(3);
  return v;
}
static std::vector<double> read_doubles(FILE* f) {
  long n = 0;
  if (fscanf(f, "%ld", &n) != 1) exit(3);
  std::vector<double> v(n);
  for (double& x : v)
    if (fscanf(f, "%lf", &x) != 1) exit(3);
  return v;
}
static bool same(const std::vector<double>& a, const std::vector<double>& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i] != b[i]) return false;
  return true;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  FILE* f = fopen(argv[1], "r");
  if (!f) return 2;
  int ncases = 0, failed = 0;
  if (fscanf(f, "%d", &ncases) != 1) return 3;
  for (int c = 0; c < ncases; ++c) {
    char kind[32];
    if (fscanf(f, "%31s", kind) != 1) return 3;
    int nthreads = 8, ierr = -1;
    const std::string k(kind);
    bool ok = false;
    if (k == "contract") {
      std::vector<int> dl = read_ints(f), ll = read_ints(f), rl = read_ints(f);
      std::vector<int> de = read_ints(f), le = read_ints(f), re = read_ints(f);
      std::vector<double> L = read_doubles(f), R = read_doubles(f), want = read_doubles(f);
      int drank = int(dl.size()), lrank = int(ll.size()), rrank = int(rl.size());
      std::vector<int> aces;
      aces.insert(aces.end(), dl.begin(), dl.end());
      aces.insert(aces.end(), ll.begin(), ll.end());
      aces.insert(aces.end(), rl.begin(), rl.end());
      std::vector<int> ptrn(lrank + rrank + 1);
      get_contraction_ptrn_(drank, lrank, rrank, aces.data(), ptrn.data(), ierr);
      std::vector<double> D(want.size(), -1.0);
      if (ierr == 0)
        tensor_block_contract__(nthreads, ptrn.data(), L.data(), lrank, le.data(), R.data(), rrank, re.data(),
                                D.data(), drank, de.data(), ierr);
      ok = ierr == 0 && same(D, want);
    } else if (k == "copy") {
      std::vector<int> ext = read_ints(f), perm = read_ints(f);  // perm: sign slot + 1-based O2N
      std::vector<double> src = read_doubles(f), want = read_doubles(f);
      int rank = int(ext.size());
      std::vector<double> out(src.size(), -1.0);
      tensor_block_copy__(nthreads, rank, ext.data(), perm.data(), src.data(), out.data(), ierr);
      ok = ierr == 0 && same(out, want);
    } else if (k == "add") {
      std::vector<int> ext = read_ints(f);
      double scale = 0.0;
      if (fscanf(f, "%lf", &scale) != 1) return 3;
      std::vector<double> t0 = read_doubles(f), t1 = read_doubles(f), want = read_doubles(f);
      int rank = int(ext.size());
      tensor_block_add__(nthreads, rank, ext.data(), t0.data(), t1.data(), scale, ierr);
      ok = ierr == 0 && same(t0, want);
    } else {
      return 3;
    }
    printf("%s %s (ierr %d)%s%s\n", kind, ok ? "ok" : "MISMATCH", ierr, ok ? "" : " ", ok ? "" : a4g_last_error());
    failed += ok ? 0 : 1;
  }
  fclose(f);
  return failed ? 1 : 0;
}
