// ref_inst.cpp -- TEST INFRASTRUCTURE ONLY (linked into oracle/_ref/ref_dump).
// Compiles the reference's scOOP/mc/paire.cpp in place and adds an explicit
// instantiation of its EPatch<WcaTruncSq> template, so that ref_dump.cpp can call
// EPatch::minDistSegments (scOOP/mc/paire.cpp:85-241) directly.
#include "mc/paire.cpp"
template class EPatch<WcaTruncSq>;
