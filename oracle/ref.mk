# Builds the reference BrainGrid single-threaded simulator from its own sources, in place where
# they lie, into oracle/_ref/ only.  This is test infrastructure (the checker), never the product.
#
#   make -f oracle/ref.mk                 # FP32 build (BGFLOAT=float)
#   make -f oracle/ref.mk fp64            # FP64 build (BGFLOAT=double)
#   make -s -f oracle/ref.mk where        # prints the reference tree used, or fails if absent
#
# The reference tree is REF, else the BRAINGRID_REF environment variable, else the checkout
# this recipe was written against; this recipe is the one place that names it.
#
# Outputs:
#   oracle/_ref/growth            unmodified driver (Core/BGDriver.cpp), XML recorder, no HDF5
#   oracle/_ref/bg_ref_harness    step-locked state dumper (oracle/ref_harness.cpp) linked to the
#                                 same reference objects
#   oracle/_ref64/...             the same two programs with BGFLOAT=double (a forced-include header
#                                 redefines the macro; the reference tree is never written)
#
# Flags follow the reference Makefile (Makefile:86): -O2 -std=c++98 -DTIXML_USE_STL -DDEBUG_OUT,
# minus the profiling/strip flags (-pg -s -g), which do not change arithmetic.

BRAINGRID_REF ?= /root/reference
REF ?= $(BRAINGRID_REF)
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT ?= $(HERE)_ref
OUT64 ?= $(HERE)_ref64
CXX ?= g++
REFFLAGS = -O2 -std=c++98 -w -DTIXML_USE_STL -DDEBUG_OUT

DIRS = Connections Core Inputs Layouts Matrix Neurons paramcontainer Recorders RNG Synapses Utils tinyxml
INC = $(addprefix -I$(REF)/,$(DIRS))

SRCS = Core/Simulator.cpp Core/SimulationInfo.cpp Core/Model.cpp \
       Layouts/Layout.cpp Layouts/FixedLayout.cpp Layouts/DynamicLayout.cpp \
       Utils/ParseParamError.cpp Utils/Timer.cpp Utils/Util.cpp Utils/Global.cpp \
       Recorders/XmlRecorder.cpp Recorders/XmlGrowthRecorder.cpp \
       Matrix/CompleteMatrix.cpp Matrix/Matrix.cpp Matrix/SparseMatrix.cpp Matrix/VectorMatrix.cpp \
       paramcontainer/ParamContainer.cpp RNG/Norm.cpp RNG/MersenneTwister.cpp \
       Core/SingleThreadedSpikingModel.cpp Core/FClassOfCategory.cpp Inputs/FSInput.cpp \
       Neurons/AllNeurons.cpp Neurons/AllSpikingNeurons.cpp Neurons/AllIFNeurons.cpp \
       Neurons/AllLIFNeurons.cpp Neurons/AllIZHNeurons.cpp \
       Synapses/AllSynapses.cpp Synapses/AllSpikingSynapses.cpp Synapses/AllDSSynapses.cpp \
       Synapses/AllSTDPSynapses.cpp Synapses/AllDynamicSTDPSynapses.cpp \
       Connections/Connections.cpp Connections/ConnGrowth.cpp Connections/ConnStatic.cpp \
       tinyxml/tinyxml.cpp tinyxml/tinyxmlparser.cpp tinyxml/tinyxmlerror.cpp tinyxml/tinystr.cpp \
       Inputs/HostSInputRegular.cpp Inputs/SInputRegular.cpp Inputs/HostSInputPoisson.cpp \
       Inputs/SInputPoisson.cpp

OBJS = $(addprefix $(OUT)/obj/,$(SRCS:.cpp=.o))
OBJS64 = $(addprefix $(OUT64)/obj/,$(SRCS:.cpp=.o))

all: $(OUT)/growth $(OUT)/bg_ref_harness
fp64: $(OUT64)/growth $(OUT64)/bg_ref_harness

$(OUT)/obj/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(REFFLAGS) $(INC) -c $< -o $@

$(OUT64)/obj/%.o: $(REF)/%.cpp $(HERE)fp64/bgfloat_double.h
	@mkdir -p $(dir $@)
	$(CXX) $(REFFLAGS) $(INC) -include $(HERE)fp64/bgfloat_double.h -c $< -o $@

$(OUT)/growth: $(OBJS) $(OUT)/obj/Core/BGDriver.o
	$(CXX) -o $@ $^

$(OUT)/bg_ref_harness: $(OBJS) $(HERE)ref_harness.cpp
	$(CXX) $(REFFLAGS) $(INC) -o $@ $(HERE)ref_harness.cpp $(OBJS)

$(OUT64)/growth: $(OBJS64) $(OUT64)/obj/Core/BGDriver.o
	$(CXX) -o $@ $^

$(OUT64)/bg_ref_harness: $(OBJS64) $(HERE)ref_harness.cpp
	$(CXX) $(REFFLAGS) $(INC) -include $(HERE)fp64/bgfloat_double.h -o $@ $(HERE)ref_harness.cpp $(OBJS64)

where:
	@test -f $(REF)/Core/BGDriver.cpp && echo $(abspath $(REF))

.PHONY: all fp64 where
