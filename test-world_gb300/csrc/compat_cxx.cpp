// compat_cxx.cpp - the drop-in entry points under the reference's C++ names.
//
// The reference declares its entry points as plain C++ functions in
// ptGraph/main.cu:30-56 (uint = unsigned int, EdgeWithWeight from
// ptGraph/globals.cuh:2-5), so a caller that keeps those prototypes links
// against C++-mangled symbols.  include/ptgraph.h exports the same functions
// with C linkage (callable from C, ctypes, cgo); this file adds the mangled
// names, each forwarding to the C symbol, so the reference's call sites link
// unchanged whether they include ptgraph.h or keep their own prototypes.
//
// It does not include ptgraph.h: the C-linkage declarations there and the
// C++ ones here have the same parameter lists, which one translation unit
// cannot hold.  The C symbols are reached through declarations whose
// assembler names are the C names (GCC/Clang asm labels).
typedef unsigned int uint;

struct EdgeWithWeight {  // ptGraph/globals.cuh:2-5 (same layout as ptg_edge_w)
    uint toNode;
    uint weight;
};

namespace ptg_c_abi {
long bfsCaculateInShare(uint, uint, uint *, uint *, uint) __asm__("bfsCaculateInShare");
long bfsCaculateInOpt(uint, uint, uint *, uint *, uint) __asm__("bfsCaculateInOpt");
long bfsCaculateInAsync(uint, uint, uint *, uint *, uint) __asm__("bfsCaculateInAsync");
long bfsCaculateInAsyncSwap(uint, uint, uint *, uint *, uint) __asm__("bfsCaculateInAsyncSwap");
long ssspCaculateInShare(uint, uint, uint *, EdgeWithWeight *, uint) __asm__("ssspCaculateInShare");
long ssspCaculateInOpt(uint, uint, uint *, EdgeWithWeight *, uint) __asm__("ssspCaculateInOpt");
long ccCaculateInShare(uint, uint, uint *, uint *) __asm__("ccCaculateInShare");
long ccCaculateInOpt(uint, uint, uint *, uint *) __asm__("ccCaculateInOpt");
long prCaculateInShare(uint, uint, uint *, uint *) __asm__("prCaculateInShare");
long prCaculateInOpt(uint, uint, uint *, uint *) __asm__("prCaculateInOpt");
void caculateInCommon(uint, uint, uint *, uint *) __asm__("caculateInCommon");
void caculateInShareOpt(uint, uint, uint *, uint *) __asm__("caculateInShareOpt");
void caculateInOptChooseByDegree(uint, uint, uint *, uint *, uint) __asm__("caculateInOptChooseByDegree");
}  // namespace ptg_c_abi

// main.cu:34-56 (caculateInOptChooseByDegree as defined at main.cu:2196-2198,
// with the source vertex; its 4-parameter declaration at main.cu:56 has no
// definition in the reference).
long bfsCaculateInShare(uint n, uint m, uint *off, uint *col, uint src) {
    return ptg_c_abi::bfsCaculateInShare(n, m, off, col, src);
}
long bfsCaculateInOpt(uint n, uint m, uint *off, uint *col, uint src) {
    return ptg_c_abi::bfsCaculateInOpt(n, m, off, col, src);
}
long bfsCaculateInAsync(uint n, uint m, uint *off, uint *col, uint src) {
    return ptg_c_abi::bfsCaculateInAsync(n, m, off, col, src);
}
long bfsCaculateInAsyncSwap(uint n, uint m, uint *off, uint *col, uint src) {
    return ptg_c_abi::bfsCaculateInAsyncSwap(n, m, off, col, src);
}
long ssspCaculateInShare(uint n, uint m, uint *off, EdgeWithWeight *edges, uint src) {
    return ptg_c_abi::ssspCaculateInShare(n, m, off, edges, src);
}
long ssspCaculateInOpt(uint n, uint m, uint *off, EdgeWithWeight *edges, uint src) {
    return ptg_c_abi::ssspCaculateInOpt(n, m, off, edges, src);
}
long ccCaculateInShare(uint n, uint m, uint *off, uint *col) { return ptg_c_abi::ccCaculateInShare(n, m, off, col); }
long ccCaculateInOpt(uint n, uint m, uint *off, uint *col) { return ptg_c_abi::ccCaculateInOpt(n, m, off, col); }
long prCaculateInShare(uint n, uint m, uint *off, uint *col) { return ptg_c_abi::prCaculateInShare(n, m, off, col); }
long prCaculateInOpt(uint n, uint m, uint *off, uint *col) { return ptg_c_abi::prCaculateInOpt(n, m, off, col); }
void caculateInCommon(uint n, uint m, uint *off, uint *col) { ptg_c_abi::caculateInCommon(n, m, off, col); }
void caculateInShareOpt(uint n, uint m, uint *off, uint *col) { ptg_c_abi::caculateInShareOpt(n, m, off, col); }
void caculateInOptChooseByDegree(uint n, uint m, uint *off, uint *col, uint src) {
    ptg_c_abi::caculateInOptChooseByDegree(n, m, off, col, src);
}
