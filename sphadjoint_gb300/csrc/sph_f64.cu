// FP64 instantiation of the engine. Compiled with --fmad=false so every
// product and sum is rounded separately, as in the reference (Julia does not
// contract a*b+c without @fastmath / @muladd): results match the oracle bit
// for bit.
#define SPH_PACK_T double
#include "sph_pack.cuh"

namespace sphgb {

FieldI *make_field_f64(const std::vector<int> &ngx, const std::vector<int> &ngy,
                         const void *host)
{
    return new Field<double>(ngx, ngy, host);
}
TapeI *make_tape_f64(int64_t N, int64_t cap, int32_t nsnap) { return new Tape<double>(N, cap, nsnap); }
StateI *make_state_f64(const std::vector<Params> &p, const std::vector<int64_t> &N, const void *X0,
                         const void *V0, NLOpts o)
{
    return new Sys<double>(p, N, X0, V0, o);
}
WorkI *make_work_f64(const std::vector<Params> &p, const std::vector<int64_t> &N)
{
    return new Work<double>(p, N);
}
PackI *make_pack_f64() { return new Packer<double>(); }

} // namespace sphgb
