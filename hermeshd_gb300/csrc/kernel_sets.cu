// kernel_sets.cu -- the launchers of one configuration (precision, basis,
// stochastic stress on/off), assembled from the instantiation units.
#include "dg_launch.cuh"

namespace hermes {
void face_f64_nb4(int, const void*, void*, const FaceArgs&, cudaStream_t);
void facen_f64_nb4(int, const void*, void*, const FaceArgs&, cudaStream_t);
void limit_f64_nb4(void*, const Geom&, const Phys&, cudaStream_t);
void mindt_f64_nb4(const void*, const DtArgs&, cudaStream_t);
void cell_f64_nb4(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
void celln_f64_nb4(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
cudaError_t prep_f64_nb4();
cudaError_t prepn_f64_nb4();
void face_f64_nb8(int, const void*, void*, const FaceArgs&, cudaStream_t);
void facen_f64_nb8(int, const void*, void*, const FaceArgs&, cudaStream_t);
void limit_f64_nb8(void*, const Geom&, const Phys&, cudaStream_t);
void mindt_f64_nb8(const void*, const DtArgs&, cudaStream_t);
void trace_f64_nb8(const void*, void*, const Geom&, cudaStream_t, int, int);
void cell_f64_nb8(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
void celln_f64_nb8(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
cudaError_t prep_f64_nb8();
cudaError_t prepn_f64_nb8();
void face_f64_nb10(int, const void*, void*, const FaceArgs&, cudaStream_t);
void facen_f64_nb10(int, const void*, void*, const FaceArgs&, cudaStream_t);
void limit_f64_nb10(void*, const Geom&, const Phys&, cudaStream_t);
void mindt_f64_nb10(const void*, const DtArgs&, cudaStream_t);
void trace_f64_nb10(const void*, void*, const Geom&, cudaStream_t, int, int);
void cell_f64_nb10(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
void celln_f64_nb10(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
cudaError_t prep_f64_nb10();
cudaError_t prepn_f64_nb10();
void face_f32_nb4(int, const void*, void*, const FaceArgs&, cudaStream_t);
void facen_f32_nb4(int, const void*, void*, const FaceArgs&, cudaStream_t);
void limit_f32_nb4(void*, const Geom&, const Phys&, cudaStream_t);
void mindt_f32_nb4(const void*, const DtArgs&, cudaStream_t);
void cell_f32_nb4(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
void celln_f32_nb4(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
cudaError_t prep_f32_nb4();
cudaError_t prepn_f32_nb4();
void face_f32_nb8(int, const void*, void*, const FaceArgs&, cudaStream_t);
void facen_f32_nb8(int, const void*, void*, const FaceArgs&, cudaStream_t);
void limit_f32_nb8(void*, const Geom&, const Phys&, cudaStream_t);
void mindt_f32_nb8(const void*, const DtArgs&, cudaStream_t);
void cell_f32_nb8(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
void celln_f32_nb8(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
cudaError_t prep_f32_nb8();
cudaError_t prepn_f32_nb8();
void face_f32_nb10(int, const void*, void*, const FaceArgs&, cudaStream_t);
void facen_f32_nb10(int, const void*, void*, const FaceArgs&, cudaStream_t);
void limit_f32_nb10(void*, const Geom&, const Phys&, cudaStream_t);
void mindt_f32_nb10(const void*, const DtArgs&, cudaStream_t);
void cell_f32_nb10(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
void celln_f32_nb10(const void*, const void*, void*, const void*, const CellArgs&, cudaStream_t);
cudaError_t prep_f32_nb10();
cudaError_t prepn_f32_nb10();

void tile_f32_nb4(const void*, const void*, void*, unsigned, const TileArgs&, cudaStream_t);
void tilen_f32_nb4(const void*, const void*, void*, unsigned, const TileArgs&, cudaStream_t);
void tile_f64_nb4(const void*, const void*, void*, unsigned, const TileArgs&, cudaStream_t);
void tilen_f64_nb4(const void*, const void*, void*, unsigned, const TileArgs&, cudaStream_t);
void dtlim_f32_nb4(void*, const DtArgs&, cudaStream_t);
void dtlim_f64_nb4(void*, const DtArgs&, cudaStream_t);
cudaError_t tprep_f32_nb4();
cudaError_t tprepn_f32_nb4();
cudaError_t tprep_f64_nb4();
cudaError_t tprepn_f64_nb4();

// the CFL reduction fused with the first stage's limiter, every instantiation
// (a small kernel, instantiated here)
static DtLimitFn dt_limit_fn(int precision, int nb) {
    if (precision == 64) return nb == 4 ? &Launch<double, 4, 2>::mindt_limit
                              : nb == 8 ? &Launch<double, 8, 2>::mindt_limit : &Launch<double, 10, 3>::mindt_limit;
    return nb == 4 ? &Launch<float, 4, 2>::mindt_limit : nb == 8 ? &Launch<float, 8, 2>::mindt_limit
                                                               : &Launch<float, 10, 3>::mindt_limit;
}

bool kernel_set(int precision, int nb, bool noise, KernelSet* out) {
    KernelSet k;
    k.mindt_limit_any = dt_limit_fn(precision, nb);
    k.trace = nullptr;
    k.tile = nullptr;
    k.mindt_limit = nullptr;
    k.prepare_tile = nullptr;
    if (precision == 64 && nb == 4) {
        k.elem_size = sizeof(double); k.nb = 4; k.nqd = 2; k.nf = 4;
        k.prepare = noise ? &prepn_f64_nb4 : &prep_f64_nb4;
        k.limit = &limit_f64_nb4;
        k.face = noise ? &facen_f64_nb4 : &face_f64_nb4;
        k.cell = noise ? &celln_f64_nb4 : &cell_f64_nb4;
        k.mindt = &mindt_f64_nb4;
        k.tile = noise ? &tilen_f64_nb4 : &tile_f64_nb4;
        k.mindt_limit = &dtlim_f64_nb4;
        k.prepare_tile = noise ? &tprepn_f64_nb4 : &tprep_f64_nb4;
        *out = k;
        return true;
    }
    if (precision == 64 && nb == 8) {
        k.elem_size = sizeof(double); k.nb = 8; k.nqd = 2; k.nf = 4;
        k.prepare = noise ? &prepn_f64_nb8 : &prep_f64_nb8;
        k.limit = &limit_f64_nb8;
        k.face = noise ? &facen_f64_nb8 : &face_f64_nb8;
        k.cell = noise ? &celln_f64_nb8 : &cell_f64_nb8;
        k.mindt = &mindt_f64_nb8;
        k.trace = noise ? nullptr : &trace_f64_nb8;
        *out = k;
        return true;
    }
    if (precision == 64 && nb == 10) {
        k.elem_size = sizeof(double); k.nb = 10; k.nqd = 3; k.nf = 9;
        k.prepare = noise ? &prepn_f64_nb10 : &prep_f64_nb10;
        k.limit = &limit_f64_nb10;
        k.face = noise ? &facen_f64_nb10 : &face_f64_nb10;
        k.cell = noise ? &celln_f64_nb10 : &cell_f64_nb10;
        k.mindt = &mindt_f64_nb10;
        k.trace = noise ? nullptr : &trace_f64_nb10;
        *out = k;
        return true;
    }
    if (precision == 32 && nb == 4) {
        k.elem_size = sizeof(float); k.nb = 4; k.nqd = 2; k.nf = 4;
        k.prepare = noise ? &prepn_f32_nb4 : &prep_f32_nb4;
        k.limit = &limit_f32_nb4;
        k.face = noise ? &facen_f32_nb4 : &face_f32_nb4;
        k.cell = noise ? &celln_f32_nb4 : &cell_f32_nb4;
        k.mindt = &mindt_f32_nb4;
        k.tile = noise ? &tilen_f32_nb4 : &tile_f32_nb4;
        k.mindt_limit = &dtlim_f32_nb4;
        k.prepare_tile = noise ? &tprepn_f32_nb4 : &tprep_f32_nb4;
        *out = k;
        return true;
    }
    if (precision == 32 && nb == 8) {
        k.elem_size = sizeof(float); k.nb = 8; k.nqd = 2; k.nf = 4;
        k.prepare = noise ? &prepn_f32_nb8 : &prep_f32_nb8;
        k.limit = &limit_f32_nb8;
        k.face = noise ? &facen_f32_nb8 : &face_f32_nb8;
        k.cell = noise ? &celln_f32_nb8 : &cell_f32_nb8;
        k.mindt = &mindt_f32_nb8;
        *out = k;
        return true;
    }
    if (precision == 32 && nb == 10) {
        k.elem_size = sizeof(float); k.nb = 10; k.nqd = 3; k.nf = 9;
        k.prepare = noise ? &prepn_f32_nb10 : &prep_f32_nb10;
        k.limit = &limit_f32_nb10;
        k.face = noise ? &facen_f32_nb10 : &face_f32_nb10;
        k.cell = noise ? &celln_f32_nb10 : &cell_f32_nb10;
        k.mindt = &mindt_f32_nb10;
        *out = k;
        return true;
    }
    return false;
}

cudaError_t adj_f64_nb4(const double*, const double*, double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t adj_f64_nb8(const double*, const double*, double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t adj_f64_nb10(const double*, const double*, double*, double*, const AdjArgs&, cudaStream_t);

cudaError_t cell_adj_dual_nb4(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t cell_adj_dual_nb8(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t cell_adj_dual_nb10(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);

cudaError_t cell_adj_rev_nb4(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t cell_adj_rev_nb8(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t cell_adj_rev_nb10(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);

cudaError_t cell_adj_rev(int nb, const double* Q, const double* mu, const double* tadj, double* out,
                         const AdjArgs& a, cudaStream_t s) {
    if (nb == 4) return cell_adj_rev_nb4(Q, mu, tadj, out, a, s);
    if (nb == 8) return cell_adj_rev_nb8(Q, mu, tadj, out, a, s);
    return cell_adj_rev_nb10(Q, mu, tadj, out, a, s);
}

cudaError_t cell_adj_gen_nb4(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t cell_adj_gen_nb8(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);
cudaError_t cell_adj_gen_nb10(const double*, const double*, const double*, double*, const AdjArgs&, cudaStream_t);

cudaError_t cell_adj_gen(int nb, const double* Q, const double* mu, const double* tadj, double* out,
                         const AdjArgs& a, cudaStream_t s) {
    if (nb == 4) return cell_adj_gen_nb4(Q, mu, tadj, out, a, s);
    if (nb == 8) return cell_adj_gen_nb8(Q, mu, tadj, out, a, s);
    return cell_adj_gen_nb10(Q, mu, tadj, out, a, s);
}

cudaError_t cell_adj_dual(int nb, const double* Q, const double* mu, const double* tadj, double* out,
                          const AdjArgs& a, cudaStream_t s) {
    if (nb == 4) return cell_adj_dual_nb4(Q, mu, tadj, out, a, s);
    if (nb == 8) return cell_adj_dual_nb8(Q, mu, tadj, out, a, s);
    return cell_adj_dual_nb10(Q, mu, tadj, out, a, s);
}

cudaError_t limit_adj_f64_nb4(const double*, const double*, double*, const Geom&, const Phys&, cudaStream_t);
cudaError_t limit_adj_f64_nb8(const double*, const double*, double*, const Geom&, const Phys&, cudaStream_t);
cudaError_t limit_adj_f64_nb10(const double*, const double*, double*, const Geom&, const Phys&, cudaStream_t);

bool limiter_adjoint_launcher(int nb, LimAdjFn* out) {
    if (nb == 4) *out = &limit_adj_f64_nb4;
    else if (nb == 8) *out = &limit_adj_f64_nb8;
    else if (nb == 10) *out = &limit_adj_f64_nb10;
    else return false;
    return true;
}

bool adjoint_launcher(int nb, AdjFn* out) {
    if (nb == 4) *out = &adj_f64_nb4;
    else if (nb == 8) *out = &adj_f64_nb8;
    else if (nb == 10) *out = &adj_f64_nb10;
    else return false;
    return true;
}
}  // namespace hermes
