# Builds the reference's own CPU path from the read-only mounted sources into
# oracle/_ref/ (git-ignored).  Used only to pin the oracle and as a CPU
# reference where the sources exist.  No cmake: g++ on the reference's worker
# sources directly, with a local stand-in for the absent OpenSSL header.
#   make -f oracle/ref.mk REF=<reference checkout> STATES=2049
ifeq ($(REF),)
$(error REF must name the reference checkout (the directory holding src/oracle.cpp))
endif
STATES ?= 2049
MAXQ ?= 32
OUT ?= oracle/_ref
CXX ?= g++
CC ?= gcc

all: $(OUT)/oracle_$(STATES) $(OUT)/compiled_$(STATES) $(OUT)/csr_ref

# The reference's randomized branching fuzz case builder and its "rf" oracle arm
# (fuzz_fullpath.cpp) behind a harness that prints per-case golden hashes.
fuzz: $(OUT)/fuzz_ref_$(STATES)

$(OUT)/sha_shim.o: oracle/ref_shim/sha256_shim.c oracle/bw_oracle.c
	mkdir -p $(OUT)
	$(CC) -O2 -c -o $(OUT)/sha_shim.o oracle/ref_shim/sha256_shim.c
	$(CC) -O2 -c -o $(OUT)/bwo.o oracle/bw_oracle.c

$(OUT)/oracle_$(STATES):
	mkdir -p $(OUT)
	$(CXX) -std=c++17 -O2 -DBWH_STATES=$(STATES) -DBWH_MAXQ=$(MAXQ) -I$(REF)/src $(REF)/src/oracle.cpp -o $@

$(OUT)/compiled_$(STATES): $(OUT)/sha_shim.o
	$(CXX) -std=c++17 -O3 -fopenmp -DBWH_STATES=$(STATES) -DBWH_MAXQ=$(MAXQ) -Ioracle/ref_shim -I$(REF)/src \
	  $(REF)/src/panel_batch_v7fix.cpp $(OUT)/sha_shim.o $(OUT)/bwo.o -o $@

# The reference's BWLEV001 event-stream emitter (emit_events.cpp), unmodified.
emit: $(OUT)/emit_events_$(STATES)

$(OUT)/emit_events_$(STATES):
	mkdir -p $(OUT)
	$(CXX) -std=c++17 -O2 -DBWH_STATES=$(STATES) -DBWH_MAXQ=$(MAXQ) -I$(REF)/src $(REF)/src/emit_events.cpp -o $@

# The reference's CsrBase rank/range (sparse_engine.hpp:70-102) behind a small harness.
$(OUT)/csr_ref: oracle/ref_csr.cpp
	mkdir -p $(OUT)
	$(CXX) -std=c++17 -O2 -fopenmp -Ioracle/ref_shim -I$(REF)/src oracle/ref_csr.cpp -o $@

$(OUT)/fuzz_ref_$(STATES): oracle/ref_fuzz.cpp $(OUT)/sha_shim.o
	$(CXX) -std=c++17 -O2 -DNDEBUG -DBWH_STATES=$(STATES) -DBWH_MAXQ=$(MAXQ) -Ioracle/ref_shim -I$(REF)/src \
	  oracle/ref_fuzz.cpp $(OUT)/bwo.o -o $@

# The reference's own GPU workers (panel_batch_gpu*.cpp, panel_gpu_session.cpp)
# compiled against this repository's include/bw_gpu.h and linked with libbwgpu.so:
# a shadow source directory of symlinks to the reference's files in which
# gpu_v7.h, gpu_v7b.h and gpu_session.h are the stand-ins of oracle/ref_shim/dropin.
PKG ?= biworlddb-artifact_gb300
CUDA ?= /usr/local/cuda
DROPIN_SRC = $(OUT)/dropin_src
DROPIN_WORKERS = panel_batch_gpu panel_batch_gpu2 panel_batch_gpu3 panel_gpu_session
dropin: $(foreach w,$(DROPIN_WORKERS),$(OUT)/$(w)_$(STATES))

$(DROPIN_SRC)/.stamp: oracle/ref_shim/dropin/gpu_v7.h oracle/ref_shim/dropin/gpu_v7b.h oracle/ref_shim/dropin/gpu_session.h
	mkdir -p $(DROPIN_SRC)
	for f in $(REF)/src/*; do case $$(basename $$f) in gpu_v7.h|gpu_v7b.h|gpu_session.h) ;; \
	  *) ln -sf $$f $(DROPIN_SRC)/ ;; esac; done
	for h in gpu_v7.h gpu_v7b.h gpu_session.h; do ln -sf $(CURDIR)/oracle/ref_shim/dropin/$$h $(DROPIN_SRC)/$$h; done
	touch $@

$(OUT)/%_$(STATES): $(DROPIN_SRC)/.stamp $(OUT)/sha_shim.o $(PKG)/libbwgpu.so
	$(CXX) -std=c++17 -O2 -w -fopenmp -DBWH_STATES=$(STATES) -DBWH_MAXQ=$(MAXQ) -Iinclude -Ioracle/ref_shim \
	  -I$(CUDA)/include $(DROPIN_SRC)/$*.cpp $(OUT)/sha_shim.o $(OUT)/bwo.o -L$(PKG) -lbwgpu \
	  -L$(CUDA)/lib64 -lcudart -Wl,-rpath,$(CURDIR)/$(PKG) -o $@

.PHONY: all fuzz dropin
