{-# LANGUAGE ForeignFunctionInterface #-}

-- | The flat scene record bling hands to the GB300 path-tracing core, and
--   its marshalling into the C ABI's structs (@include/bling_gpu.h@).
--
--   bling's 'Scene', 'Primitive' and 'Material' are closures
--   (@Scene.hs:20-26@, @Primitive.hs:21-27@, @Reflection.hs:42@) and cannot
--   cross an FFI, so the parser state (@IO/ParserCore.hs:45-58@) records this
--   flat description beside them as it builds primitives:
--
--   * 'PState' gains @flat :: FlatScene@ and @flatMaterial :: FlatMaterial@
--     (the flat twin of @material@, set by @pMaterial@) and
--     @flatEmit :: Maybe [Float]@ (the twin of @emit@);
--   * @prim { mesh ... }@ conses a 'FlatMesh' with the world-space vertices
--     @mkTriangleMesh@ computes (@TriangleMesh.hs:56-59@), and
--     @prim { shape ... }@ a 'FlatShape' with the transform and emission,
--     both with the index of 'flatMaterial' in 'fsMaterials' -- consed, as
--     @object@ prepends @prims@ (@IO/RenderJob.hs:52@), so 'fsPrims' keeps
--     the primitive order @mkScene@ hands to @mkKdTree@ (@Scene.hs:37-43@);
--   * @light { ... }@ conses a 'FlatLight', and @camera { ... }@ sets
--     'fsCamera' from @mkProjective@'s matrices (@Camera.hs:108-135@).
--
--   Every 'Storable' instance takes its offsets and sizes from the C header
--   through hsc2hs, so the record follows the header field for field.
--   Compile with @hsc2hs -I include@ (cabal: @build-tools: hsc2hs@,
--   @include-dirs: include@).
module Graphics.Bling.IO.GpuScene (
   -- * The flat scene
   FlatScene(..), FlatPrim(..), FlatMesh(..), FlatShape(..), FlatMaterial(..),
   FlatLight(..), FlatCamera(..), FlatTexture(..), emptyFlatScene,

   -- * Marshalling
   SceneDesc, RenderParams(..), withSceneDesc, withRenderParams,
   abiVersion, bands
   ) where

import           Control.Monad (forM_, zipWithM_)
import           Data.Int
import           Data.Word
import qualified Data.Vector.Storable as SV
import           Foreign
import           Foreign.C.Types

#include "bling_gpu.h"

-- | @BLING_ABI_VERSION@ of the header this module was compiled against;
--   compare it with @bling_abi_version()@ once at start-up
abiVersion :: Int
abiVersion = #{const BLING_ABI_VERSION}

-- | spectral bands per spectrum (@BLING_BANDS@, 'Spectrum' of Spectrum.hs)
bands :: Int
bands = #{const BLING_BANDS}

--------------------------------------------------------------------------------
-- The flat record
--------------------------------------------------------------------------------

-- | @bling_material@: kind (@BLING_MAT_*@), scalars and 16-band spectra;
--   the diffuse colour of matte, plastic and substrate may be a checker
--   board or graph paper of two spectra (@kd_texture@, @kd_tex_params@,
--   @kd2@).  Any parameter may instead name a texture of 'fsTextures'
--   ('fmTex', slot @BLING_SLOT_*@, node index + 1, 0 for the constant), and
--   'fmBump' the displacement of @bumpMapped@ (node index + 1, or 0)
data FlatMaterial = FlatMaterial
   { fmKind        :: !Int32
   , fmSigma       :: !Float
   , fmRoughness   :: !Float
   , fmIor         :: !Float
   , fmKd          :: ![Float]
   , fmKs          :: ![Float]
   , fmKt          :: ![Float]
   , fmEta         :: ![Float]
   , fmK           :: ![Float]
   , fmKdTexture   :: !Int32
   , fmKdTexParams :: ![Float]   -- ^ 9 entries
   , fmKd2         :: ![Float]
   , fmTex         :: ![Int32]   -- ^ 8 entries
   , fmBump        :: !Int32
   } deriving (Show, Eq)

-- | @bling_texture@: one node of a texture expression (@BLING_TEXN_*@),
--   its children by index into 'fsTextures' (each before its parent), the
--   mapping, its numbers, and the pixels of an image (8-bit RGB or grey,
--   rows top to bottom) or the steps of a gradient (position and spectrum,
--   17 floats each)
data FlatTexture = FlatTexture
   { ftKind     :: !Int32
   , ftChildren :: !(Int32, Int32, Int32)
   , ftIValue   :: !Int32
   , ftMapKind  :: !Int32
   , ftMap      :: ![Float]  -- ^ 16 entries
   , ftP        :: ![Float]  -- ^ 4 entries
   , ftSpectrum :: ![Float]
   , ftSteps    :: !(Maybe (SV.Vector Float))
   , ftPixels   :: !(Maybe (Int32, Int32, SV.Vector Word8))
   } deriving (Show, Eq)

-- | @bling_mesh_desc@: world-space vertices (3 per vertex), indices (a
--   multiple of 3), optional normals and uvs, a material index
data FlatMesh = FlatMesh
   { fmeshVertices :: !(SV.Vector Float)
   , fmeshIndices  :: !(SV.Vector Int32)
   , fmeshNormals  :: !(Maybe (SV.Vector Float))
   , fmeshUVs      :: !(Maybe (SV.Vector Float))
   , fmeshMaterial :: !Int32
   } deriving (Show, Eq)

-- | @bling_shape_desc@: @BLING_SHAPE_*@, up to 6 parameters, object-to-world
--   and its inverse (row major, the 'Transform' pair of Transform.hs),
--   material index and the emission of an area light
data FlatShape = FlatShape
   { fsKind     :: !Int32
   , fsParams   :: ![Float]
   , fsO2W      :: ![Float]
   , fsW2O      :: ![Float]
   , fsMaterial :: !Int32
   , fsEmission :: !(Maybe [Float])
   } deriving (Show, Eq)

-- | a primitive, in primitive-list order
data FlatPrim = PrimMesh !FlatMesh | PrimShape !FlatShape deriving (Show, Eq)

-- | @bling_light_desc@: directional, point, infinite (with its lat-long
--   map of @envW * envH * 16@ floats and world-to-light transform pair) or
--   sun/sky (@mkSunSkyLight east sunDir turbidity@: sun direction in
--   'flVec', 'flEast', 'flTurbidity')
data FlatLight = FlatLight
   { flKind      :: !Int32
   , flSpectrum  :: ![Float]
   , flVec       :: ![Float]
   , flEnv       :: !(Maybe (Int32, Int32, SV.Vector Float))
   , flW2L       :: ![Float]
   , flL2W       :: ![Float]
   , flEast      :: ![Float]
   , flTurbidity :: !Float
   } deriving (Show, Eq)

-- | @bling_camera_desc@: the matrices of 'ProjectiveCamera' (Camera.hs:24-31)
data FlatCamera = FlatCamera
   { fcC2W       :: ![Float]
   , fcC2WInv    :: ![Float]
   , fcR2C       :: ![Float]
   , fcR2CInv    :: ![Float]
   , fcLensR     :: !Float
   , fcFocalD    :: !Float
   , fcW2R       :: ![Float]
   , fcPixelArea :: !Float
   } deriving (Show, Eq)

data FlatScene = FlatScene
   { fsMaterials :: ![FlatMaterial]  -- ^ indexed by the primitives' material
   , fsTextures  :: ![FlatTexture]   -- ^ indexed by the materials' 'fmTex' and 'fmBump'
   , fsPrims     :: ![FlatPrim]      -- ^ newest first, as @prims@ of PState
   , fsLights    :: ![FlatLight]     -- ^ newest first, as @lights@ of PState
   , fsCamera    :: !FlatCamera
   } deriving (Show, Eq)

emptyFlatScene :: FlatCamera -> FlatScene
emptyFlatScene = FlatScene [] [] [] []

--------------------------------------------------------------------------------
-- Storable instances of the fixed-size records
--------------------------------------------------------------------------------

-- | writes exactly n floats (the list padded with zeros)
pokeFloats :: Ptr a -> Int -> [Float] -> IO ()
pokeFloats p n xs = pokeArray (castPtr p :: Ptr CFloat) (map realToFrac $ take n (xs ++ repeat 0))

peekFloats :: Ptr a -> Int -> IO [Float]
peekFloats p n = map realToFrac <$> peekArray n (castPtr p :: Ptr CFloat)

instance Storable FlatMaterial where
   sizeOf _ = #{size bling_material}
   alignment _ = #{alignment bling_material}
   poke p m = do
      #{poke bling_material, kind} p (fmKind m)
      #{poke bling_material, sigma} p (CFloat $ fmSigma m)
      #{poke bling_material, roughness} p (CFloat $ fmRoughness m)
      #{poke bling_material, ior} p (CFloat $ fmIor m)
      pokeFloats (#{ptr bling_material, kd} p) bands (fmKd m)
      pokeFloats (#{ptr bling_material, ks} p) bands (fmKs m)
      pokeFloats (#{ptr bling_material, kt} p) bands (fmKt m)
      pokeFloats (#{ptr bling_material, eta} p) bands (fmEta m)
      pokeFloats (#{ptr bling_material, k} p) bands (fmK m)
      #{poke bling_material, kd_texture} p (fmKdTexture m)
      pokeFloats (#{ptr bling_material, kd_tex_params} p) 9 (fmKdTexParams m)
      pokeFloats (#{ptr bling_material, kd2} p) bands (fmKd2 m)
      pokeArray (#{ptr bling_material, tex} p) (take 8 (fmTex m ++ repeat 0))
      #{poke bling_material, bump} p (fmBump m)
      #{poke bling_material, reserved_tex} p (0 :: Int32)
   peek p = FlatMaterial
      <$> #{peek bling_material, kind} p
      <*> (unF <$> #{peek bling_material, sigma} p)
      <*> (unF <$> #{peek bling_material, roughness} p)
      <*> (unF <$> #{peek bling_material, ior} p)
      <*> peekFloats (#{ptr bling_material, kd} p) bands
      <*> peekFloats (#{ptr bling_material, ks} p) bands
      <*> peekFloats (#{ptr bling_material, kt} p) bands
      <*> peekFloats (#{ptr bling_material, eta} p) bands
      <*> peekFloats (#{ptr bling_material, k} p) bands
      <*> #{peek bling_material, kd_texture} p
      <*> peekFloats (#{ptr bling_material, kd_tex_params} p) 9
      <*> peekFloats (#{ptr bling_material, kd2} p) bands
      <*> peekArray 8 (#{ptr bling_material, tex} p)
      <*> #{peek bling_material, bump} p

unF :: CFloat -> Float
unF = realToFrac

instance Storable FlatShape where
   sizeOf _ = #{size bling_shape_desc}
   alignment _ = #{alignment bling_shape_desc}
   poke p s = do
      #{poke bling_shape_desc, kind} p (fsKind s)
      #{poke bling_shape_desc, material} p (fsMaterial s)
      pokeFloats (#{ptr bling_shape_desc, params} p) 6 (fsParams s)
      pokeFloats (#{ptr bling_shape_desc, o2w} p) 16 (fsO2W s)
      pokeFloats (#{ptr bling_shape_desc, w2o} p) 16 (fsW2O s)
      #{poke bling_shape_desc, emissive} p (maybe 0 (const 1) (fsEmission s) :: Int32)
      pokeFloats (#{ptr bling_shape_desc, emission} p) bands (maybe [] id (fsEmission s))
   peek p = do
      e <- #{peek bling_shape_desc, emissive} p :: IO Int32
      em <- peekFloats (#{ptr bling_shape_desc, emission} p) bands
      FlatShape
         <$> #{peek bling_shape_desc, kind} p
         <*> peekFloats (#{ptr bling_shape_desc, params} p) 6
         <*> peekFloats (#{ptr bling_shape_desc, o2w} p) 16
         <*> peekFloats (#{ptr bling_shape_desc, w2o} p) 16
         <*> #{peek bling_shape_desc, material} p
         <*> pure (if e /= 0 then Just em else Nothing)

instance Storable FlatCamera where
   sizeOf _ = #{size bling_camera_desc}
   alignment _ = #{alignment bling_camera_desc}
   poke p c = do
      pokeFloats (#{ptr bling_camera_desc, c2w} p) 16 (fcC2W c)
      pokeFloats (#{ptr bling_camera_desc, c2w_inv} p) 16 (fcC2WInv c)
      pokeFloats (#{ptr bling_camera_desc, r2c} p) 16 (fcR2C c)
      pokeFloats (#{ptr bling_camera_desc, r2c_inv} p) 16 (fcR2CInv c)
      #{poke bling_camera_desc, lens_radius} p (CFloat $ fcLensR c)
      #{poke bling_camera_desc, focal_distance} p (CFloat $ fcFocalD c)
      pokeFloats (#{ptr bling_camera_desc, w2r} p) 16 (fcW2R c)
      #{poke bling_camera_desc, pixel_area} p (CFloat $ fcPixelArea c)
      #{poke bling_camera_desc, reserved} p (0 :: CFloat)
   peek p = FlatCamera
      <$> peekFloats (#{ptr bling_camera_desc, c2w} p) 16
      <*> peekFloats (#{ptr bling_camera_desc, c2w_inv} p) 16
      <*> peekFloats (#{ptr bling_camera_desc, r2c} p) 16
      <*> peekFloats (#{ptr bling_camera_desc, r2c_inv} p) 16
      <*> (unF <$> #{peek bling_camera_desc, lens_radius} p)
      <*> (unF <$> #{peek bling_camera_desc, focal_distance} p)
      <*> peekFloats (#{ptr bling_camera_desc, w2r} p) 16
      <*> (unF <$> #{peek bling_camera_desc, pixel_area} p)

-- | @bling_render_params@ (64 bytes)
data RenderParams = RenderParams
   { rpWidth, rpHeight     :: !Int32
   , rpStrataX, rpStrataY  :: !Int32
   , rpMaxDepth            :: !Int32
   , rpSampleDepth         :: !Int32
   , rpRRDepth             :: !Int32   -- ^ 7 in the reference (Path.hs:68)
   , rpFilterKind          :: !Int32
   , rpFilterParams        :: ![Float] -- ^ 4 entries
   , rpSeed                :: !Word64
   , rpSamplerKind         :: !Int32
   } deriving (Show, Eq)

instance Storable RenderParams where
   sizeOf _ = #{size bling_render_params}
   alignment _ = #{alignment bling_render_params}
   poke p r = do
      #{poke bling_render_params, width} p (rpWidth r)
      #{poke bling_render_params, height} p (rpHeight r)
      #{poke bling_render_params, strata_x} p (rpStrataX r)
      #{poke bling_render_params, strata_y} p (rpStrataY r)
      #{poke bling_render_params, max_depth} p (rpMaxDepth r)
      #{poke bling_render_params, sample_depth} p (rpSampleDepth r)
      #{poke bling_render_params, rr_depth} p (rpRRDepth r)
      #{poke bling_render_params, filter_kind} p (rpFilterKind r)
      pokeFloats (#{ptr bling_render_params, filter_params} p) 4 (rpFilterParams r)
      #{poke bling_render_params, seed} p (rpSeed r)
      #{poke bling_render_params, sampler_kind} p (rpSamplerKind r)
      #{poke bling_render_params, reserved} p (0 :: Int32)
   peek p = RenderParams
      <$> #{peek bling_render_params, width} p
      <*> #{peek bling_render_params, height} p
      <*> #{peek bling_render_params, strata_x} p
      <*> #{peek bling_render_params, strata_y} p
      <*> #{peek bling_render_params, max_depth} p
      <*> #{peek bling_render_params, sample_depth} p
      <*> #{peek bling_render_params, rr_depth} p
      <*> #{peek bling_render_params, filter_kind} p
      <*> peekFloats (#{ptr bling_render_params, filter_params} p) 4
      <*> #{peek bling_render_params, seed} p
      <*> #{peek bling_render_params, sampler_kind} p

withRenderParams :: RenderParams -> (Ptr RenderParams -> IO a) -> IO a
withRenderParams = with

--------------------------------------------------------------------------------
-- The scene descriptor: arrays of records that point into Haskell vectors
--------------------------------------------------------------------------------

-- | the C @bling_scene_desc@ (only ever handled through a pointer)
data SceneDesc

-- | keeps the storable vectors of a mesh pinned while the callback runs
withVec :: Storable a => Maybe (SV.Vector a) -> (Ptr a -> IO b) -> IO b
withVec Nothing f = f nullPtr
withVec (Just v) f = SV.unsafeWith v f

withMeshes :: [FlatMesh] -> ([(FlatMesh, Ptr Float, Ptr Int32, Ptr Float, Ptr Float)] -> IO a)
           -> IO a
withMeshes [] k = k []
withMeshes (m:ms) k =
   SV.unsafeWith (fmeshVertices m) $ \pv ->
   SV.unsafeWith (fmeshIndices m) $ \pi' ->
   withVec (fmeshNormals m) $ \pn ->
   withVec (fmeshUVs m) $ \pu ->
   withMeshes ms $ \rest -> k ((m, pv, pi', pn, pu) : rest)

withEnvs :: [FlatLight] -> ([Ptr Float] -> IO a) -> IO a
withEnvs [] k = k []
withEnvs (l:ls) k = withVec (fmap (\(_, _, v) -> v) (flEnv l)) $ \pe ->
   withEnvs ls $ \rest -> k (pe : rest)

pokeMesh :: Ptr () -> (FlatMesh, Ptr Float, Ptr Int32, Ptr Float, Ptr Float) -> IO ()
pokeMesh p (m, pv, pi', pn, pu) = do
   #{poke bling_mesh_desc, vertices} p pv
   #{poke bling_mesh_desc, n_vertices} p (fromIntegral (SV.length (fmeshVertices m) `div` 3) :: Int64)
   #{poke bling_mesh_desc, indices} p pi'
   #{poke bling_mesh_desc, n_indices} p (fromIntegral (SV.length (fmeshIndices m)) :: Int64)
   #{poke bling_mesh_desc, normals} p pn
   #{poke bling_mesh_desc, uvs} p pu
   #{poke bling_mesh_desc, material} p (fmeshMaterial m)
   #{poke bling_mesh_desc, reserved} p (0 :: Int32)

withTextures :: [FlatTexture] -> ([(FlatTexture, Ptr Float, Ptr Word8)] -> IO a) -> IO a
withTextures [] k = k []
withTextures (t:ts) k =
   withVec (ftSteps t) $ \ps ->
   withVec (fmap (\(_, _, v) -> v) (ftPixels t)) $ \px ->
   withTextures ts $ \rest -> k ((t, ps, px) : rest)

pokeTexture :: Ptr () -> (FlatTexture, Ptr Float, Ptr Word8) -> IO ()
pokeTexture p (t, ps, px) = do
   let (a, b, c) = ftChildren t
   #{poke bling_texture, kind} p (ftKind t)
   #{poke bling_texture, a} p a
   #{poke bling_texture, b} p b
   #{poke bling_texture, c} p c
   #{poke bling_texture, ivalue} p (ftIValue t)
   #{poke bling_texture, map_kind} p (ftMapKind t)
   pokeFloats (#{ptr bling_texture, map} p) 16 (ftMap t)
   pokeFloats (#{ptr bling_texture, p} p) 4 (ftP t)
   pokeFloats (#{ptr bling_texture, spectrum} p) bands (ftSpectrum t)
   #{poke bling_texture, data} p ps
   #{poke bling_texture, pixels} p px
   #{poke bling_texture, width} p (maybe 0 (\(w, _, _) -> w) (ftPixels t))
   #{poke bling_texture, height} p (maybe 0 (\(_, h, _) -> h) (ftPixels t))

pokeLight :: Ptr () -> (FlatLight, Ptr Float) -> IO ()
pokeLight p (l, pe) = do
   #{poke bling_light_desc, kind} p (flKind l)
   pokeFloats (#{ptr bling_light_desc, spectrum} p) bands (flSpectrum l)
   pokeFloats (#{ptr bling_light_desc, vec} p) 3 (flVec l)
   #{poke bling_light_desc, env} p pe
   #{poke bling_light_desc, env_w} p (maybe 0 (\(w, _, _) -> w) (flEnv l))
   #{poke bling_light_desc, env_h} p (maybe 0 (\(_, h, _) -> h) (flEnv l))
   pokeFloats (#{ptr bling_light_desc, w2l} p) 16 (flW2L l)
   pokeFloats (#{ptr bling_light_desc, l2w} p) 16 (flL2W l)
   pokeFloats (#{ptr bling_light_desc, east} p) 3 (flEast l)
   #{poke bling_light_desc, turbidity} p (CFloat $ flTurbidity l)

-- | Lays the flat scene out as a @bling_scene_desc@ for the duration of the
--   callback (for @bling_scene_create@, which copies everything it needs).
--   Primitive IDs: meshes and shapes in 'fsPrims' order, which is already
--   the reference's primitive order; lights in the order of 'fsLights'.
withSceneDesc :: FlatScene -> (Ptr SceneDesc -> IO a) -> IO a
withSceneDesc sc k =
   withMeshes meshes $ \ms ->
   withEnvs (fsLights sc) $ \envs ->
   withTextures (fsTextures sc) $ \txs ->
   allocaBytes (max 1 (length txs) * #{size bling_texture}) $ \pTex ->
   allocaBytes (max 1 (length ms) * #{size bling_mesh_desc}) $ \pMeshes ->
   allocaArray (max 1 (length shapes)) $ \pShapes ->
   allocaArray (max 1 (length (fsMaterials sc))) $ \pMats ->
   allocaBytes (max 1 (length (fsLights sc)) * #{size bling_light_desc}) $ \pLights ->
   withArray (if null order then [0] else order) $ \pOrder ->
   allocaBytes #{size bling_scene_desc} $ \d -> do
      forM_ (zip [0 ..] ms) $ \(i, m) ->
         pokeMesh (pMeshes `plusPtr` (i * #{size bling_mesh_desc})) m
      pokeArray pShapes shapes
      pokeArray pMats (fsMaterials sc)
      zipWithM_ (\i le -> pokeLight (pLights `plusPtr` (i * #{size bling_light_desc})) le)
                [0 ..] (zip (fsLights sc) envs)
      zipWithM_ (\i t -> pokeTexture (pTex `plusPtr` (i * #{size bling_texture})) t) [0 ..] txs
      #{poke bling_scene_desc, meshes} d pMeshes
      #{poke bling_scene_desc, n_meshes} d (fromIntegral (length ms) :: Int32)
      #{poke bling_scene_desc, shapes} d pShapes
      #{poke bling_scene_desc, n_shapes} d (fromIntegral (length shapes) :: Int32)
      #{poke bling_scene_desc, materials} d pMats
      #{poke bling_scene_desc, n_materials} d (fromIntegral (length (fsMaterials sc)) :: Int32)
      #{poke bling_scene_desc, lights} d pLights
      #{poke bling_scene_desc, n_lights} d (fromIntegral (length (fsLights sc)) :: Int32)
      #{poke bling_scene_desc, prim_order} d pOrder
      #{poke bling_scene_desc, camera} d (fsCamera sc)
      #{poke bling_scene_desc, textures} d pTex
      #{poke bling_scene_desc, n_textures} d (fromIntegral (length txs) :: Int32)
      #{poke bling_scene_desc, reserved_desc} d (0 :: Int32)
      k (castPtr d)
   where
      meshes = [m | PrimMesh m <- fsPrims sc]
      shapes = [s | PrimShape s <- fsPrims sc]
      -- v >= 0: mesh v; v < 0: shape (complement v), in primitive order
      order = go (0 :: Int32) (0 :: Int32) (fsPrims sc)
      go _ _ [] = []
      go mi si (PrimMesh _ : ps) = mi : go (mi + 1) si ps
      go mi si (PrimShape _ : ps) = complement si : go mi (si + 1) ps
