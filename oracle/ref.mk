# Builds the reference's own `red` executable (its FP64 CPU path, `red -cpu`) from
# the unmodified reference sources, for use as a cross-check of the C restatement in
# this directory. Outputs go to oracle/_ref/ only (git-ignored).
#
#   make -f oracle/ref.mk REF=/root/reference -j8
#
# Three build shims are applied from the command line, never by editing sources:
#  * cudaDeviceProp::clockRate no longer exists in CUDA 13 (used only in a device
#    query printout, util.cu:86) -> the token is mapped onto another int member;
#  * options.cpp uses fabs without <cmath> -> force-include it in the plain C++ files;
#  * int_rungekutta5.cu does not compile against integrator.h (its constructor has a
#    different signature, int_rungekutta5.cu:96 vs integrator.h:20) and the reference
#    refuses to create it anyway (options.cpp:252-255) -> it is left out.
# Host code is built with -ffp-contract=off so that the CPU path evaluates every
# expression operation by operation (the reference builds with -fmad=false, Makefile:17;
# gcc on aarch64 would otherwise contract a*b+c into fma).

REF      ?= /root/reference
OUT      := oracle/_ref
SRC      := $(REF)/red.cuda/src
RED      := $(SRC)/red.cuda
UTIL     := $(SRC)/red.cuda.utility
ARCH     ?= -gencode arch=compute_103a,code=sm_103a
NVFLAGS  := -O2 -fmad=false $(ARCH) -I$(REF)/red.cuda/red.type -I$(UTIL) \
            -DclockRate=major -Xcompiler -ffp-contract=off -w
CXXFLAGS := -O2 -ffp-contract=off -w -include cmath -I$(REF)/red.cuda/red.type -I$(UTIL) \
            -I$(CUDA_HOME)/include
CUDA_HOME ?= /usr/local/cuda

RED_SRCS := gas_disk.cpp integrator.cu nbody_exception.cpp number_of_bodies.cpp \
            options.cpp parameter.cpp tokenizer.cpp int_euler.cu int_rungekutta2.cu \
            int_rungekutta4.cu int_rungekutta8.cu main.cu pp_disk.cu
UTIL_SRCS := file_util.cpp tools.cpp util.cu

RED_OBJS  := $(addprefix $(OUT)/obj/red_,$(addsuffix .o,$(basename $(RED_SRCS))))
UTIL_OBJS := $(addprefix $(OUT)/obj/util_,$(addsuffix .o,$(basename $(UTIL_SRCS))))

all: $(OUT)/red

$(OUT)/red: $(RED_OBJS) $(UTIL_OBJS)
	nvcc $(ARCH) -o $@ $^

$(OUT)/obj/red_%.o: $(RED)/%.cu | $(OUT)/obj
	nvcc $(NVFLAGS) -x cu -c $< -o $@
$(OUT)/obj/red_%.o: $(RED)/%.cpp | $(OUT)/obj
	g++ $(CXXFLAGS) -c $< -o $@
$(OUT)/obj/util_%.o: $(UTIL)/%.cu | $(OUT)/obj
	nvcc $(NVFLAGS) -x cu -c $< -o $@
$(OUT)/obj/util_%.o: $(UTIL)/%.cpp | $(OUT)/obj
	g++ $(CXXFLAGS) -c $< -o $@

$(OUT)/obj:
	mkdir -p $@

.PHONY: all
