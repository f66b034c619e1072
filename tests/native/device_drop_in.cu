// A user translation unit written against the reference's device API
// (namespace cuda, rns_const_init), compiled with include/grns/device.cuh in
// place of the reference's headers.  The moduli set comes from a params.h
// pre-included on the command line.  Driven by tests/test_gpu_device_header.py.
#include <cstdint>

#include "grns/device.cuh"

constexpr int NM = RNS_MODULI_SIZE;

__global__ void k_user(int count, const int *x, const int *y, const int *d, const unsigned *D, er_float_t *ev,
                       int *cmp, int *q, int *r, int *sc, mp_int_t *ma, mp_int_t *mb, mp_int_t *mm) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int xs[NM], ys[NM], ds[NM], qs[NM], rs[NM], ss[NM];
    for (int i = 0; i < NM; i++) {
        xs[i] = x[k * NM + i];
        ys[i] = y[k * NM + i];
        ds[i] = d[k * NM + i];
    }
    cuda::rns_eval_compute(&ev[2 * k], &ev[2 * k + 1], xs);
    cmp[k] = cuda::rns_cmp(xs, ys);
    cuda::rns_div(qs, rs, xs, ds);
    cuda::rns_scale2pow(ss, xs, D[k]);
    for (int i = 0; i < NM; i++) {
        q[k * NM + i] = qs[i];
        r[k * NM + i] = rs[i];
        sc[k * NM + i] = ss[i];
    }
    cuda::mpint_mul(&mm[k], &ma[k], &mb[k]);
}

template <class T>
static int to_dev(T **d, const T *h, size_t n) {
    if (cudaMalloc(d, n * sizeof(T)) != cudaSuccess) return 1;
    return h && cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess;
}

/* runs k_user on host arrays (AoS residues); returns 0 on success */
extern "C" int run_user_kernel(int count, const int *x, const int *y, const int *d, const unsigned *D,
                               er_float_t *ev, int *cmp, int *q, int *r, int *sc, const mp_int_t *ma,
                               const mp_int_t *mb, mp_int_t *mm) {
    rns_const_init();
    mpint_const_init();
    if (grns_device_init_status() != cudaSuccess) return 2;
    const size_t rn = (size_t)count * NM;
    int *dx, *dy, *dd, *dcmp, *dq, *dr, *dsc;
    unsigned *dD;
    er_float_t *dev;
    mp_int_t *dma, *dmb, *dmm;
    if (to_dev(&dx, x, rn) || to_dev(&dy, y, rn) || to_dev(&dd, d, rn) || to_dev(&dD, D, (size_t)count) ||
        to_dev(&dev, (const er_float_t *)nullptr, 2 * (size_t)count) || to_dev(&dcmp, (const int *)nullptr, count) ||
        to_dev(&dq, (const int *)nullptr, rn) || to_dev(&dr, (const int *)nullptr, rn) ||
        to_dev(&dsc, (const int *)nullptr, rn) || to_dev(&dma, ma, count) || to_dev(&dmb, mb, count) ||
        to_dev(&dmm, (const mp_int_t *)nullptr, count))
        return 3;
    k_user<<<(count + 127) / 128, 128>>>(count, dx, dy, dd, dD, dev, dcmp, dq, dr, dsc, dma, dmb, dmm);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    cudaMemcpy(ev, dev, 2 * (size_t)count * sizeof(er_float_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(cmp, dcmp, (size_t)count * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(q, dq, rn * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(r, dr, rn * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(sc, dsc, rn * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(mm, dmm, (size_t)count * sizeof(mp_int_t), cudaMemcpyDeviceToHost);
    for (void *p : {(void *)dx, (void *)dy, (void *)dd, (void *)dD, (void *)dev, (void *)dcmp, (void *)dq, (void *)dr,
                    (void *)dsc, (void *)dma, (void *)dmb, (void *)dmm})
        cudaFree(p);
    return cudaGetLastError() != cudaSuccess ? 5 : 0;
}
