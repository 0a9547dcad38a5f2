"""The LCA module (input -> residual <-> V1) as an OpenPV params file, for the host column tests:
the topology of the LCA tutorials -- IdentConn input -> residual (channel 0), HyPerConn
V1 -> residual (channel 1, presynaptic perspective, V1 sparse), TransposeConn residual -> V1
(postsynaptic perspective) -- with the delivery switches as arguments."""


def lca_params(nb=2, n=32, c=1, v1_scale=0.5, nf=16, nxp=8, vthresh=0.1, tau=100.0, receive_gpu=False,
               sparse=True, post_perspective=True, err_scale=1.0, v1_keyword="HyPerLCALayer", momentum=0.0):
    rg = "true" if receive_gpu else "false"
    return f"""
// LCA module: input -> residual <-> V1
debugParsing = false;

HyPerCol "column" = {{
   nx = {n};
   ny = {n};
   nbatch = {nb};
   dt = 1.0;
   stopTime = 100;
   progressInterval = 10;
}};

ImageLayer "Input" = {{
   nxScale = 1;
   nyScale = 1;
   nf = {c};
   phase = 0;
   displayPeriod = 0;
   inputPath = "input/frames.txt";
}};

ANNErrorLayer "Residual" = {{
   nxScale = 1;
   nyScale = 1;
   nf = {c};
   phase = 1;
   errScale = {err_scale};
   VThresh = -infinity;
   sparseLayer = false;
}};

{v1_keyword} "V1" = {{
   LCAMomentumRate = {momentum};
   nxScale = {v1_scale};
   nyScale = {v1_scale};
   nf = {nf};
   phase = 2;
   InitVType = "ZeroV";
   timeConstantTau = {tau};
   selfInteract = true;
   VThresh = {vthresh};
   AMin = 0;
   AMax = infinity;
   AShift = {vthresh};
   VWidth = 0;
   sparseLayer = {"true" if sparse else "false"};
}};

IdentConn "InputToResidual" = {{
   preLayerName = "Input";
   postLayerName = "Residual";
   channelCode = 0;
   delay = [0.000000];
}};

HyPerConn "V1ToResidual" = {{
   preLayerName = "V1";
   postLayerName = "Residual";
   channelCode = 1;
   nxp = {nxp};
   nyp = {nxp};
   nfp = {c};
   sharedWeights = true;
   weightInitType = "FileWeight";
   initWeightsFile = "input/dictionary.pvp";
   plasticityFlag = false;
   receiveGpu = {rg};
   updateGSynFromPostPerspective = false;
   pvpatchAccumulateType = "convolve";
}};

TransposeConn "ResidualToV1" = {{
   preLayerName = "Residual";
   postLayerName = "V1";
   channelCode = 0;
   originalConnName = "V1ToResidual";
   receiveGpu = {rg};
   updateGSynFromPostPerspective = {"true" if post_perspective else "false"};
   pvpatchAccumulateType = "convolve";
}};
"""
