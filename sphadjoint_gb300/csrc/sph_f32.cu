// FP32 instantiation of the engine: same kernels, multiply-add contraction on
// (checked against the FP64 oracle within a relative tolerance).
#define SPH_PACK_T float
#include "sph_pack.cuh"

namespace sphgb {

FieldI *make_field_f32(const std::vector<int> &ngx, const std::vector<int> &ngy,
                         const void *host)
{
    return new Field<float>(ngx, ngy, host);
}
TapeI *make_tape_f32(int64_t N, int64_t cap, int32_t nsnap) { return new Tape<float>(N, cap, nsnap); }
StateI *make_state_f32(const std::vector<Params> &p, const std::vector<int64_t> &N, const void *X0,
                         const void *V0, NLOpts o)
{
    return new Sys<float>(p, N, X0, V0, o);
}
WorkI *make_work_f32(const std::vector<Params> &p, const std::vector<int64_t> &N)
{
    return new Work<float>(p, N);
}
PackI *make_pack_f32() { return new Packer<float>(); }

} // namespace sphgb
