# Builds the reference's own driver with the GPU model replaced by this drop-in:
#
#   make -f braingrid_gb300/dropin/dropin.mk [REF=<reference tree>]
#
# Core/BGDriver.cpp and every host source the reference's GPU build links (Makefile:96-160 of the
# reference: the model, neuron, synapse, connection, layout, recorder, input, matrix, RNG,
# parameter and tinyxml sources) are compiled unmodified from the reference tree, in place where
# they lie, with the reference's flags plus -DUSE_GPU (Makefile:86-87), into
# braingrid_gb300/_build/dropin/ only.  None of the reference's CUDA translation units
# (Core/GPUSpikingModel.cu, Neurons/*_d.cu, Synapses/*_d.cu, Connections/ConnGrowth_d.cu,
# Inputs/Gpu*.cu, RNG/MersenneTwister_d.cu) and none of its NVIDIA sample files (Utils/Book.h,
# RNG/MersenneTwister_d.*) is compiled or linked: the three files of this directory define what
# they defined, on libbg3.so.  The host-only stimulus classes (Inputs/HostSInput*.cpp) are not
# part of a GPU build (Inputs/FSInput.cpp picks the Gpu* classes under USE_GPU).
#
# Output: braingrid_gb300/_build/dropin/growth_bg3 (linked to braingrid_gb300/_build/libbg3.so,
# found at run time next to it through the executable's RPATH).  The reference tree is REF, else
# the one oracle/ref.mk resolves.

HERE := $(dir $(lastword $(MAKEFILE_LIST)))
ROOT := $(abspath $(HERE)/../..)
REF ?= $(shell make -s -f $(ROOT)/oracle/ref.mk where)
OUT := $(ROOT)/braingrid_gb300/_build/dropin
LIBDIR := $(ROOT)/braingrid_gb300/_build
CUDA ?= /usr/local/cuda
CXX ?= g++

# the reference's headers are C++98 (in-class float constants), so this directory's files are too
REFFLAGS = -O2 -std=c++98 -w -DTIXML_USE_STL -DDEBUG_OUT -DUSE_GPU
OURFLAGS = -O2 -std=c++98 -ffp-contract=off -Wall -Wno-unused-parameter -DTIXML_USE_STL -DDEBUG_OUT -DUSE_GPU

DIRS = Connections Core Inputs Layouts Matrix Neurons paramcontainer Recorders RNG Synapses Utils tinyxml
INC = $(addprefix -I$(REF)/,$(DIRS))

SRCS = Core/BGDriver.cpp Core/Simulator.cpp Core/SimulationInfo.cpp Core/Model.cpp \
       Core/FClassOfCategory.cpp \
       Layouts/Layout.cpp Layouts/FixedLayout.cpp Layouts/DynamicLayout.cpp \
       Utils/ParseParamError.cpp Utils/Timer.cpp Utils/Util.cpp Utils/Global.cpp \
       Recorders/XmlRecorder.cpp Recorders/XmlGrowthRecorder.cpp \
       Matrix/CompleteMatrix.cpp Matrix/Matrix.cpp Matrix/SparseMatrix.cpp Matrix/VectorMatrix.cpp \
       paramcontainer/ParamContainer.cpp RNG/Norm.cpp RNG/MersenneTwister.cpp \
       Inputs/FSInput.cpp Inputs/SInputRegular.cpp Inputs/SInputPoisson.cpp \
       Neurons/AllNeurons.cpp Neurons/AllSpikingNeurons.cpp Neurons/AllIFNeurons.cpp \
       Neurons/AllLIFNeurons.cpp Neurons/AllIZHNeurons.cpp \
       Synapses/AllSynapses.cpp Synapses/AllSpikingSynapses.cpp Synapses/AllDSSynapses.cpp \
       Synapses/AllSTDPSynapses.cpp Synapses/AllDynamicSTDPSynapses.cpp \
       Connections/Connections.cpp Connections/ConnGrowth.cpp Connections/ConnStatic.cpp \
       tinyxml/tinyxml.cpp tinyxml/tinyxmlparser.cpp tinyxml/tinyxmlerror.cpp tinyxml/tinystr.cpp
OURS = GPUSpikingModel.cpp bg3_classes.cpp GpuSInput.cpp

OBJS = $(addprefix $(OUT)/ref/,$(SRCS:.cpp=.o))
OUROBJS = $(addprefix $(OUT)/,$(OURS:.cpp=.o))

all: $(OUT)/growth_bg3

$(OUT)/ref/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(REFFLAGS) $(INC) -c $< -o $@

$(OUT)/%.o: $(HERE)%.cpp $(HERE)bg3_dropin.h $(ROOT)/include/bg3.h
	@mkdir -p $(OUT)
	$(CXX) $(OURFLAGS) -I$(HERE) -I$(ROOT)/include $(INC) -c $< -o $@

# every symbol resolved at link time (an executable link fails on any undefined reference);
# libbg3.so's own dependencies (the CUDA runtime) resolve through its DT_NEEDED entries
$(OUT)/growth_bg3: $(OBJS) $(OUROBJS) $(LIBDIR)/libbg3.so
	$(CXX) -o $@ $(OBJS) $(OUROBJS) -L$(LIBDIR) -lbg3 -Wl,-rpath,'$$ORIGIN/..' \
	    -Wl,-rpath-link,$(CUDA)/lib64 -Wl,--no-allow-shlib-undefined -L$(CUDA)/lib64

.PHONY: all
