// engine_u32.cu — suffix-sort engine instantiated for uint32_t symbols.
#include "engine_impl.cuh"

namespace capssa {
capssa_status engine_build_u32(Ctx &c, const EngineArgs &a) { return engine_build_t<uint32_t>(c, a); }
}  // namespace capssa
