// A caller of the reference's C++ interface, unchanged in form: it includes
// gpu_pcg.cuh and calls solvePCG<T> / pcg_solve<T> with host arrays, as
// examples/pcg_solve.cu of the reference does.  Inputs come from a binary file
// written by tests/test_cpp_dropin_gpu.py:
//   uint32 n, N, dtype(4|8), with_pinv; then S (3n^2N), Pinv (3n^2N, if any),
//   gamma (nN), lambda0 (nN).  with_pinv = 2 passes S and Pinv as csr_t (the
//   reference's CSR overload of solvePCG), built here from the cbtd arrays.
// Output (stdout): "iters <k>" then the solution as hex of its bytes.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "gpu_pcg.cuh"

// cbtd (n x 3n column-major block row per knot) -> CSR of the n N x n N matrix
template <typename T>
struct HostCsr {
    std::vector<uint32_t> row_ptr, col_ind;
    std::vector<T> val;
    csr_t<T> csr;
};

template <typename T>
void to_csr(const std::vector<T> &M, uint32_t n, uint32_t N, HostCsr<T> &out) {
    out.row_ptr.assign(1, 0);
    for (uint32_t r = 0; r < n * N; ++r) {
        const uint32_t k = r / n, i = r % n;
        for (uint32_t b = 0; b < 3; ++b) {
            if ((b == 0 && k == 0) || (b == 2 && k + 1 == N)) continue;
            const uint32_t kc = k + b - 1;
            for (uint32_t j = 0; j < n; ++j) {
                const T v = M[(size_t)k * 3 * n * n + (size_t)(b * n + j) * n + i];
                if (v != T(0)) {
                    out.col_ind.push_back(kc * n + j);
                    out.val.push_back(v);
                }
            }
        }
        out.row_ptr.push_back((uint32_t)out.col_ind.size());
    }
    out.csr = csr_t<T>{out.row_ptr.data(), out.col_ind.data(), out.val.data(), n * N, n * N,
                       (uint32_t)out.val.size()};
}

template <typename T>
int run(FILE *f, uint32_t n, uint32_t N, uint32_t with_pinv, uint32_t max_iter, double tol) {
    const size_t mat = (size_t)3 * n * n * N, vec = (size_t)n * N;
    std::vector<T> S(mat), P(with_pinv ? mat : 0), g(vec), lam(vec);
    if (fread(S.data(), sizeof(T), mat, f) != mat) return 2;
    if (with_pinv && fread(P.data(), sizeof(T), mat, f) != mat) return 2;
    if (fread(g.data(), sizeof(T), vec, f) != vec) return 2;
    if (fread(lam.data(), sizeof(T), vec, f) != vec) return 2;
    pcg_config<T> config((T)tol, max_iter);
    uint32_t iters;
    if (with_pinv == 2) {
        HostCsr<T> cS, cP;
        to_csr(S, n, N, cS);
        to_csr(P, n, N, cP);
        iters = solvePCG<T>(&cS.csr, &cP.csr, g.data(), lam.data(), n, N, &config);
    } else if (with_pinv)
        iters = solvePCG<T>(S.data(), P.data(), g.data(), lam.data(), n, N, &config);
    else
        iters = (uint32_t)pcg_solve<T>(S.data(), g.data(), lam.data(), n, N, &config);
    printf("iters %u\n", iters);
    const unsigned char *b = reinterpret_cast<const unsigned char *>(lam.data());
    for (size_t i = 0; i < vec * sizeof(T); ++i) printf("%02x", b[i]);
    printf("\n");
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 4) return 1;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 1;
    uint32_t hdr[4];
    if (fread(hdr, sizeof(uint32_t), 4, f) != 4) return 2;
    const uint32_t max_iter = (uint32_t)atoi(argv[2]);
    const double tol = atof(argv[3]);
    const int rc = hdr[2] == 8 ? run<double>(f, hdr[0], hdr[1], hdr[3], max_iter, tol)
                               : run<float>(f, hdr[0], hdr[1], hdr[3], max_iter, tol);
    fclose(f);
    return rc;
}
