// ref_gene_qc.cpp -- host build of the reference's gene QC tool.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile (target `ref`) into
// the executable oracle/_ref/gene_qc_ref from the reference's own sources where
// they lie under REF_ROOT: tools/gene_qc.cpp unchanged, on top of the
// reference's src/api/api.cpp built with its CPU shim (whose align_sw_batch
// runs the reference's SW trace kernel on the host).  Nothing of the reference
// is copied here.  tests/golden/make_gene_qc_golden.py runs it to write the
// gene QC fixtures; it is never part of the product.
#define GENOALIGNER_HIP_SHIM 1
#include "src/api/api.cpp"
#include "tools/gene_qc.cpp"
