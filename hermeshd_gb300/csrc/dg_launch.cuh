// dg_launch.cuh -- host-side launchers of the stage kernels for one
// (T, NB, NQD) instantiation, collected in a KernelSet so the C-ABI layer can
// pick the instantiation at context creation.  Each inst_*.cu file compiles
// one instantiation (the files build in parallel).
#pragma once

#include <cuda_runtime.h>

#include "dg_kernels.cuh"

namespace hermes {

struct KernelSet {
    int elem_size;
    int nb, nqd, nf;
    cudaError_t (*prepare)();
    void (*limit)(void* Q, const Geom& G, const Phys& ph, cudaStream_t s);
    void (*face)(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s);
    void (*cell)(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s);
    void (*mindt)(const void* Q, const DtArgs& a, cudaStream_t s);
};

template <class T, int NB, int NQD>
struct Launch {
    using TB = hermes_tab::Tab<NB, NQD>;
    static size_t cell_smem() { return (size_t)2 * NB * NQ * CELL_TPB * sizeof(T); }
    static cudaError_t prepare() {
        return cudaFuncSetAttribute(k_cell<T, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cell_smem());
    }
    static void limit(void* Q, const Geom& G, const Phys& ph, cudaStream_t s) {
        if (G.ncell <= 0) return;
        const unsigned nb = (unsigned)((G.ncell + LIMIT_TPB - 1) / LIMIT_TPB);
        k_limit<T, TB><<<nb, LIMIT_TPB, 0, s>>>(static_cast<T*>(Q), G, ph);
    }
    static void face(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s) {
        const long long n = a.G.nface[dir];
        if (n <= 0) return;
        dim3 grid((unsigned)((n + FACE_TPB - 1) / FACE_TPB), TB::NF);
        const T* q = static_cast<const T*>(Q);
        T* f = static_cast<T*>(flux);
        if (dir == 0) k_face<T, TB, 0><<<grid, FACE_TPB, 0, s>>>(q, f, a);
        else if (dir == 1) k_face<T, TB, 1><<<grid, FACE_TPB, 0, s>>>(q, f, a);
        else k_face<T, TB, 2><<<grid, FACE_TPB, 0, s>>>(q, f, a);
    }
    static void cell(const void* Qin, const void* Q0, void* out, const void* flux, const CellArgs& a, cudaStream_t s) {
        if (a.G.ncell <= 0) return;
        const unsigned nb = (unsigned)((a.G.ncell + CELL_TPB - 1) / CELL_TPB);
        k_cell<T, TB><<<nb, CELL_TPB, cell_smem(), s>>>(static_cast<const T*>(Qin), static_cast<const T*>(Q0),
                                                        static_cast<T*>(out), static_cast<const T*>(flux), a);
    }
    static void mindt(const void* Q, const DtArgs& a, cudaStream_t s) {
        if (a.G.ncell <= 0) return;
        const unsigned nb = (unsigned)((a.G.ncell + DT_TPB - 1) / DT_TPB);
        k_mindt<T><<<nb, DT_TPB, 0, s>>>(static_cast<const T*>(Q), a);
    }
    static KernelSet set() {
        KernelSet k;
        k.elem_size = sizeof(T);
        k.nb = NB; k.nqd = NQD; k.nf = TB::NF;
        k.prepare = &prepare;
        k.limit = &limit;
        k.face = nullptr;   // set by the cell translation unit
        k.cell = &cell;
        k.mindt = &mindt;
        return k;
    }
};

// one per inst_<type>_nb<N>_cell.cu; the face launcher of the same
// instantiation lives in inst_<type>_nb<N>_face.cu so the two halves compile
// in parallel
#define HERMES_DECLARE_INST(TN, NBV)                                                            \
    KernelSet kernels_##TN##_nb##NBV();                                                         \
    void face_##TN##_nb##NBV(int dir, const void* Q, void* flux, const FaceArgs& a, cudaStream_t s);
HERMES_DECLARE_INST(f64, 4)
HERMES_DECLARE_INST(f64, 8)
HERMES_DECLARE_INST(f64, 10)
HERMES_DECLARE_INST(f32, 4)
HERMES_DECLARE_INST(f32, 8)
HERMES_DECLARE_INST(f32, 10)

}  // namespace hermes
