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

/* the other serial functions: mp_int division, mixed-radix digits, their comparison, rns_div_fast */
__global__ void k_user2(int count, const int *x, const int *y, const int *d, mp_int_t *ma, mp_int_t *mb,
                        mp_int_t *md, int *mr, int *mcmp, int *q, int *r) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int xs[NM], ys[NM], ds[NM], a[NM], qs[NM], rs[NM];
    for (int i = 0; i < NM; i++) {
        xs[i] = x[k * NM + i];
        ys[i] = y[k * NM + i];
        ds[i] = d[k * NM + i];
    }
    cuda::mpint_div(&md[k], &ma[k], &mb[k]);
    cuda::mrc(a, xs);
    mcmp[k] = cuda::mrc_compare_rns(xs, ys);
    cuda::rns_div_fast(qs, rs, xs, ds);
    for (int i = 0; i < NM; i++) {
        mr[k * NM + i] = a[i];
        q[k * NM + i] = qs[i];
        r[k * NM + i] = rs[i];
    }
}

/* the n-threaded forms: one block of NM threads per number, operands in global memory */
__global__ void k_user_par(const int *x, const int *y, const int *d, er_float_t *ev, int *cmp, int *q, int *r,
                           int *mr, int *msd, int *mcmp) {
    const int k = blockIdx.x;
    int *xk = const_cast<int *>(x) + k * NM, *yk = const_cast<int *>(y) + k * NM, *dk = const_cast<int *>(d) + k * NM;
    cuda::rns_eval_compute_parallel(&ev[2 * k], &ev[2 * k + 1], xk);
    const int c = cuda::rns_cmp_parallel(xk, yk);
    if (threadIdx.x == 0) cmp[k] = c;
    cuda::rns_div_parallel(q + k * NM, r + k * NM, xk, dk);
    cuda::mrc_pipeline(mr + k * NM, xk);
    const int m = cuda::mrc_pipeline_msd(xk);
    if (threadIdx.x == 0) msd[k] = m;
    const int mc = cuda::mrc_pipeline_compare_rns(xk, yk);
    if (threadIdx.x == 0) mcmp[k] = mc;
}

template <class T>
static int to_dev(T **d, const T *h, size_t n) {
    if (cudaMalloc(d, n * sizeof(T)) != cudaSuccess) return 1;
    return h && cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess;
}

/* runs k_user on host arrays (AoS residues); returns 0 on success */
extern "C" __attribute__((visibility("default"))) int run_user_kernel(int count, const int *x, const int *y, const int *d, const unsigned *D,
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

template <class T>
static void back(T *h, const T *d, size_t n) {
    cudaMemcpy(h, d, n * sizeof(T), cudaMemcpyDeviceToHost);
}

/* k_user2 and k_user_par on host arrays; returns 0 on success */
extern "C" __attribute__((visibility("default"))) int run_user_kernel2(int count, const int *x, const int *y, const int *d, const mp_int_t *ma,
                                const mp_int_t *mb, mp_int_t *md, int *mr, int *mcmp, int *q, int *r,
                                er_float_t *pev, int *pcmp, int *pq, int *pr, int *pmr, int *pmsd, int *pmcmp) {
    rns_const_init();
    if (grns_device_init_status() != cudaSuccess) return 2;
    const size_t rn = (size_t)count * NM;
    int *dx, *dy, *dd, *dmr, *dmc, *dq, *dr, *dpc, *dpq, *dpr, *dpm, *dps, *dpmc;
    mp_int_t *dma, *dmb, *dmd;
    er_float_t *dpe;
    if (to_dev(&dx, x, rn) || to_dev(&dy, y, rn) || to_dev(&dd, d, rn) || to_dev(&dma, ma, count) ||
        to_dev(&dmb, mb, count) || to_dev(&dmd, (const mp_int_t *)nullptr, count) ||
        to_dev(&dmr, (const int *)nullptr, rn) || to_dev(&dmc, (const int *)nullptr, count) ||
        to_dev(&dq, (const int *)nullptr, rn) || to_dev(&dr, (const int *)nullptr, rn) ||
        to_dev(&dpe, (const er_float_t *)nullptr, 2 * (size_t)count) || to_dev(&dpc, (const int *)nullptr, count) ||
        to_dev(&dpq, (const int *)nullptr, rn) || to_dev(&dpr, (const int *)nullptr, rn) ||
        to_dev(&dpm, (const int *)nullptr, rn) || to_dev(&dps, (const int *)nullptr, count) ||
        to_dev(&dpmc, (const int *)nullptr, count))
        return 3;
    k_user2<<<(count + 127) / 128, 128>>>(count, dx, dy, dd, dma, dmb, dmd, dmr, dmc, dq, dr);
    k_user_par<<<count, NM>>>(dx, dy, dd, dpe, dpc, dpq, dpr, dpm, dps, dpmc);
    if (cudaDeviceSynchronize() != cudaSuccess) return 4;
    back(md, dmd, count);
    back(mr, dmr, rn);
    back(mcmp, dmc, count);
    back(q, dq, rn);
    back(r, dr, rn);
    back(pev, dpe, 2 * (size_t)count);
    back(pcmp, dpc, count);
    back(pq, dpq, rn);
    back(pr, dpr, rn);
    back(pmr, dpm, rn);
    back(pmsd, dps, count);
    back(pmcmp, dpmc, count);
    for (void *p : {(void *)dx, (void *)dy, (void *)dd, (void *)dma, (void *)dmb, (void *)dmd, (void *)dmr,
                    (void *)dmc, (void *)dq, (void *)dr, (void *)dpe, (void *)dpc, (void *)dpq, (void *)dpr,
                    (void *)dpm, (void *)dps, (void *)dpmc})
        cudaFree(p);
    return cudaGetLastError() != cudaSuccess ? 5 : 0;
}
