# icl_sampo.mk - builds the reference's own host program, src/abms.c,
# unmodified, over icl_sampo.cpp and libsampo_cuda.so: the SAMPO command
# line and output files with the hourly loop on the GPU.
#
#   make -f sampo_gb300/host/icl_sampo.mk SAMPO=<the SAMPO checkout> [OUT=<dir>]
#   (build libsampo_cuda.so first: python -m sampo_gb300.build)
#
# -> $(OUT)/abms_gb300, run as the reference's bin/abms:
#   cd <run dir> && $(OUT)/abms_gb300 temp.txt environment.txt [species.h]
HERE := $(abspath $(dir $(lastword $(MAKEFILE_LIST))))
REPO := $(abspath $(HERE)/../..)
ifndef SAMPO
$(error set SAMPO to the SAMPO checkout whose src/abms.c and include/ to build)
endif
OUT ?= $(REPO)/sampo_gb300/_build/icl
LIBDIR := $(REPO)/sampo_gb300/_build
INC := -I$(HERE)/cl_types -I$(SAMPO)/include -I$(REPO)/include
FP := -O2 -ffp-contract=off

all: $(OUT)/abms_gb300

$(OUT):
	mkdir -p $(OUT)
$(OUT)/abms.o: $(SAMPO)/src/abms.c | $(OUT)
	gcc $(FP) -std=gnu99 -fms-extensions -w $(INC) -c $< -o $@
$(OUT)/icl_sampo.o: $(HERE)/icl_sampo.cpp $(REPO)/include/sampo.h | $(OUT)
	g++ $(FP) -std=c++17 -Wall -Wno-unused-result $(INC) -c $< -o $@
$(OUT)/abms_gb300: $(OUT)/abms.o $(OUT)/icl_sampo.o $(LIBDIR)/libsampo_cuda.so
	g++ -o $@ $(OUT)/abms.o $(OUT)/icl_sampo.o -L$(LIBDIR) -lsampo_cuda -Wl,-rpath,$(LIBDIR) -lm

clean:
	rm -f $(OUT)/abms.o $(OUT)/icl_sampo.o $(OUT)/abms_gb300
.PHONY: all clean
